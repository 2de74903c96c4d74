// bella_expl3d.cu -- the explicit parts of the 3D projection on the device:
// euler_forward_non_advective (second_projection.py:22-74, with the 2D branch's
// glue: the divergence on node.isc) and euler_backward_non_advective_expl_part
// (:77-92).  The arithmetic is bella_expl3d.cuh's (checked on the CPU by
// tests/test_expl3d_host.py); boundary data are the advection's boundary lines
// (bella_advect.cuh), which restate set_explicit_boundary_data axis by axis.
//   k_e3_zero_ghost   divergence_nodes' y-wall ghost momenta            :542-551
//   k_e3_fw_nodes     divergence, wall doubling, pressure increment     :39-47, :66
//   k_e3_fw_cells     momenta and rhoX from the old p2                   :49-64
//   k_e3_fw_p2        p2 += compressibility * increment                  :68-69
//   k_e3_ghost        ghost nodes of p2 along one axis                   :71
//   k_e3_xp_cells     buoyancy, wind, Coriolis inverse                   :82-90
//   k_e3_bd           boundary data along one axis                       :72, :92
#include "bella_advect.cuh"
#include "bella_expl3d.cuh"
#include "bella_internal.cuh"

namespace bella {

__global__ void k_e3_zero_ghost(Expl3Geom G, Expl3Fields F) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)G.icx * G.icz || G.bc[1] != 1) return;
    const int i = (int)(e / G.icz), k = (int)(e - (long long)i * G.icz);
    const int rows[4] = {0, 1, G.icy - 2, G.icy - 1};
    for (int t = 0; t < 4; ++t) {
        const long long c = e3_cell(G, i, rows[t], k);
        F.f[1][c] = 0.0;
        F.f[2][c] = 0.0;
        F.f[3][c] = 0.0;
    }
}

__global__ void k_e3_fw_nodes(Expl3Geom G, Expl3Fields F, double *rhs, double *dp) {
    const int nx = G.icx - 1, ny = G.icy - 1, nz = G.icz - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nx * ny * nz) return;
    const int a = (int)(e / ((long long)ny * nz));
    const int r = (int)(e - (long long)a * ny * nz);
    const int b = r / nz, c = r - b * nz;
    double inc;
    const double div = e3_forward_node(G, a, b, c, F, &inc);
    if (rhs) rhs[e] = div;
    dp[e] = inc;
}

__global__ void k_e3_fw_cells(Expl3Geom G, Expl3Fields F, const double *p2, const double *S0c, const double *S0n) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)G.icx * G.icy * G.icz) return;
    const int i = (int)(e / ((long long)G.icy * G.icz));
    const int r = (int)(e - (long long)i * G.icy * G.icz);
    const int j = r / G.icz, k = r - j * G.icz;
    e3_forward_cell(G, i, j, k, p2, S0c, S0n, F);
}

__global__ void k_e3_fw_p2(Expl3Geom G, const double *dp, double *p2) {
    const int nx = G.icx - 1, ny = G.icy - 1, nz = G.icz - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nx * ny * nz) return;
    const int a = (int)(e / ((long long)ny * nz));
    const int r = (int)(e - (long long)a * ny * nz);
    const int b = r / nz, c = r - b * nz;
    const long long n = e3_node(G, a + 1, b + 1, c + 1);
    p2[n] += G.compressibility * dp[e];
}

__global__ void k_e3_ghost(Expl3Geom G, int d, double *p) {
    const int nn[3] = {G.icx + 1, G.icy + 1, G.icz + 1};
    const long long nl = (long long)nn[d == 0 ? 1 : 0] * nn[d == 2 ? 1 : 2];
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l < nl) e3_ghost_line(G, d, l, p);
}

__global__ void k_e3_xp_cells(Expl3Geom G, Expl3Fields F, const double *S0n) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)G.icx * G.icy * G.icz) return;
    const int j = (int)((e / G.icz) % G.icy);
    e3_expl_part_cell(G, e, j, S0n, F);
}

__global__ void k_e3_bd(AdvGeom A, int s, AdvFields F, const double *rhoY0, const double *strat_inv) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < adv_nl(A, s)) adv_bd_line(A, s, l, F, rhoY0, strat_inv);
}

namespace {

int nblk(long long n) { return (int)((n + 255) / 256); }

bool e3_setup(const bella_expl3d *a, Expl3Geom &G, Expl3Fields &F, AdvGeom &A, AdvFields &AF) {
    if (!a || a->inx < 5 || a->iny < 5 || a->inz < 5) return false;
    const double *req[] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->S0n, a->hydro_rhoY0,
                           a->strat_inv};
    for (const double *p : req)
        if (!p) return false;
    G.icx = a->inx + 3; G.icy = a->iny + 3; G.icz = a->inz + 3;
    G.bc[0] = a->x_wall ? 1 : 0; G.bc[1] = a->y_wall ? 1 : 0; G.bc[2] = a->z_wall ? 1 : 0;
    G.dx = a->dx; G.dy = a->dy; G.dz = a->dz; G.dt = a->dt;
    G.Msq = a->Msq; G.g = a->g; G.gamm = a->gamm; G.nonhydro = a->nonhydro; G.compressibility = a->compressibility;
    for (int q = 0; q < 3; ++q) {
        G.cor[q] = a->coriolis[q];
        G.wind[q] = a->wind[q];
    }
    G.is_ArakawaKonor = a->is_ArakawaKonor;
    G.xsign = a->div_sign_2d ? 1.0 : -1.0;
    double *f[6] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX};
    for (int q = 0; q < 6; ++q) F.f[q] = AF.f[q] = f[q];
    A.nd = 3;
    A.ic[0] = G.icx; A.ic[1] = G.icy; A.ic[2] = G.icz;
    for (int q = 0; q < 3; ++q) A.bc[q] = G.bc[q];
    A.d[0] = a->dx; A.d[1] = a->dy; A.d[2] = a->dz;
    A.g = a->g; A.gamm = a->gamm; A.is_compressible = a->is_compressible;
    return true;
}

void e3_boundary(const AdvGeom &A, const AdvFields &AF, const bella_expl3d *a, cudaStream_t s) {
    for (int d = 0; d < 3; ++d) k_e3_bd<<<nblk(adv_nl(A, d)), 256, 0, s>>>(A, d, AF, a->hydro_rhoY0, a->strat_inv);
}

}  // namespace
}  // namespace bella

using namespace bella;

extern "C" int bella_euler_forward3d(const bella_expl3d *a, void *stream) {
    Expl3Geom G;
    Expl3Fields F;
    AdvGeom A;
    AdvFields AF;
    if (!e3_setup(a, G, F, A, AF) || !a->p2 || !a->S0c || !a->scratch) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    const long long nisc = (long long)(G.icx - 1) * (G.icy - 1) * (G.icz - 1);
    const long long ncell = (long long)G.icx * G.icy * G.icz;
    k_e3_zero_ghost<<<nblk((long long)G.icx * G.icz), 256, 0, s>>>(G, F);
    k_e3_fw_nodes<<<nblk(nisc), 256, 0, s>>>(G, F, a->rhs_out, a->scratch);
    k_e3_fw_cells<<<nblk(ncell), 256, 0, s>>>(G, F, a->p2, a->S0c, a->S0n);
    k_e3_fw_p2<<<nblk(nisc), 256, 0, s>>>(G, a->scratch, a->p2);
    const long long nn[3] = {(long long)G.icx + 1, (long long)G.icy + 1, (long long)G.icz + 1};
    for (int d = 0; d < 3; ++d)
        k_e3_ghost<<<nblk(nn[d == 0 ? 1 : 0] * nn[d == 2 ? 1 : 2]), 256, 0, s>>>(G, d, a->p2);
    e3_boundary(A, AF, a, s);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" int bella_expl_part3d(const bella_expl3d *a, void *stream) {
    Expl3Geom G;
    Expl3Fields F;
    AdvGeom A;
    AdvFields AF;
    if (!e3_setup(a, G, F, A, AF)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    k_e3_xp_cells<<<nblk((long long)G.icx * G.icy * G.icz), 256, 0, s>>>(G, F, a->S0n);
    e3_boundary(A, AF, a, s);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}
