// bella_adv2d.cu -- the 2D advection of the reference (explicit.py, recovery.py,
// numerical_flux.py) on the device: face mass fluxes, the Strang-split sweeps of
// advect and the first-order advect_rk.
//
// The arithmetic lives in bella_adv2d.cuh (host/device functions, checked on the
// CPU against the reference by tests/test_adv2d_host.py); each kernel here runs
// one of those functions for every line, face or cell of a sweep:
//   k_adv_bd       boundary data along the sweep axis, one thread per line
//   k_adv_faces    recovery + upwind flux of one inner face per thread
//   k_adv_update   conservative update, one thread per cell
//   k_adv_pwchi    rhoX update of advect_rk's y sweep
//   k_adv_mass     face mass fluxes rhoY u / rhoY v, one thread per inner face
// The sweeps are bandwidth-trivial next to the projection's solve; no sweep
// reads what its own launch writes (faces read cells, updates read faces).
#include "bella_adv2d.cuh"
#include "bella_internal.cuh"

namespace bella {

__global__ void k_adv_bd(AdvGeom G, int s, AdvFields F, const double *rhoY0, const double *strat_inv) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < adv_nl(G, s)) adv_bd_line(G, s, l, F, rhoY0, strat_inv);
}

__global__ void k_adv_faces(AdvGeom G, int s, AdvFields F, double lmbda, AdvFaces out) {
    const int nf = adv_ns(G, s) - 1;                          // inner faces 1 .. ns-1 of a line
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)adv_nl(G, s) * nf) return;
    const int l = (int)(e / nf), f = 1 + (int)(e - (long long)l * nf);
    adv_face_flux(G, s, l, f, F, lmbda, out);
}

__global__ void k_adv_update(AdvGeom G, int s, AdvFields F, AdvFaces fl, double lmbda) {
    const int ns = adv_ns(G, s);
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)adv_nl(G, s) * ns) return;
    const int l = (int)(e / ns), c = (int)(e - (long long)l * ns);
    adv_update_cell(G, s, l, c, F, fl, lmbda);
}

__global__ void k_adv_pwchi(AdvGeom G, AdvFaces fy, double lmbda, double *pw) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)G.icx * G.icy) return;
    const int l = (int)(e / G.icy), c = (int)(e - (long long)l * G.icy);
    pw[adv_cell(G, 1, l, c)] = lmbda * (fy.f[5][adv_face(G, 1, l, c)] - fy.f[5][adv_face(G, 1, l, c + 1)]);
}

__global__ void k_adv_mass(AdvGeom G, AdvFields F, double *fx_rhoY, double *fy_rhoY) {
    const long long nx = (long long)(G.icy - 2) * (G.icx - 1);   // x faces: rows 1..icy-2, faces 1..icx-1
    const long long ny = (long long)(G.icx - 2) * (G.icy - 1);   // y faces: columns 1..icx-2, faces 1..icy-1
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e < nx) {
        const int j = 1 + (int)(e / (G.icx - 1)), f = 1 + (int)(e % (G.icx - 1));
        fx_rhoY[adv_face(G, 0, j, f)] = adv_mass_x(G, F, j, f);
    } else if (e < nx + ny) {
        const long long r = e - nx;
        const int i = 1 + (int)(r / (G.icy - 1)), f = 1 + (int)(r % (G.icy - 1));
        fy_rhoY[adv_face(G, 1, i, f)] = adv_mass_y(G, F, i, f);
    }
}

namespace {

int blocks(long long n) { return (int)((n + 255) / 256); }

struct DevEx {
    AdvGeom G;
    AdvFields F;
    AdvFaces fl[2];
    const double *rhoY0, *strat_inv;
    double *pw;
    cudaStream_t st;
    void bd(int s) {
        k_adv_bd<<<blocks(adv_nl(G, s)), 256, 0, st>>>(G, s, F, rhoY0, strat_inv);
    }
    void faces(int s, double lmbda) {
        k_adv_faces<<<blocks((long long)adv_nl(G, s) * (adv_ns(G, s) - 1)), 256, 0, st>>>(G, s, F, lmbda, fl[s]);
    }
    void update(int s, double lmbda) {
        k_adv_update<<<blocks((long long)adv_nl(G, s) * adv_ns(G, s)), 256, 0, st>>>(G, s, F, fl[s], lmbda);
    }
    void pwchi(double lmbda) {
        if (!pw) return;
        k_adv_pwchi<<<blocks((long long)G.icx * G.icy), 256, 0, st>>>(G, fl[1], lmbda, pw);
    }
};

bool adv_setup(const bella_adv2d *a, DevEx &ex, void *stream) {
    if (!a || a->inx < 5 || a->iny < 5) return false;
    const double *req[] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0, a->strat_inv};
    for (const double *p : req)
        if (!p) return false;
    for (int q = 0; q < 6; ++q)
        if (!a->fx[q] || !a->fy[q]) return false;
    ex.G.icx = a->inx + 3; ex.G.icy = a->iny + 3;
    ex.G.bc[0] = a->x_wall ? 1 : 0; ex.G.bc[1] = a->y_wall ? 1 : 0;
    ex.G.dx = a->dx; ex.G.dy = a->dy; ex.G.g = a->g; ex.G.gamm = a->gamm; ex.G.is_compressible = a->is_compressible;
    double *f[6] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX};
    for (int q = 0; q < 6; ++q) {
        ex.F.f[q] = f[q];
        ex.fl[0].f[q] = a->fx[q];
        ex.fl[1].f[q] = a->fy[q];
    }
    ex.rhoY0 = a->hydro_rhoY0; ex.strat_inv = a->strat_inv; ex.pw = a->pwchi;
    ex.st = (cudaStream_t)stream;
    return true;
}

}  // namespace
}  // namespace bella

using namespace bella;

extern "C" int bella_advective_fluxes2d(const bella_adv2d *a, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    const long long n = (long long)(ex.G.icy - 2) * (ex.G.icx - 1) + (long long)(ex.G.icx - 2) * (ex.G.icy - 1);
    k_adv_mass<<<blocks(n), 256, 0, ex.st>>>(ex.G, ex.F, a->fx[4], a->fy[4]);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" int bella_advect2d(const bella_adv2d *a, double dt, int odd, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    adv_strang(ex, ex.G, dt, odd);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" int bella_advect_rk2d(const bella_adv2d *a, double dt, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    adv_rk(ex, ex.G, dt);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// set_explicit_boundary_data (boundary.py:7-216) of the whole state: x, then y
extern "C" int bella_boundary2d(const bella_adv2d *a, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    ex.bd(0);
    ex.bd(1);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}
