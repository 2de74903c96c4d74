// bella_advect.cu -- the advection of the reference (explicit.py, recovery.py,
// numerical_flux.py) on the device, 2D and 3D: face mass fluxes, the Strang-split
// sweeps of advect and the first-order advect_rk.
//
// The arithmetic lives in bella_advect.cuh (host/device functions, checked on the
// CPU against the reference by tests/test_advect_host.py); each kernel here runs
// one of those functions for every line, face or cell of a sweep:
//   k_adv_bd       boundary data along the sweep axis, one thread per line
//   k_adv_faces    recovery + upwind flux of one inner face per thread
//   k_adv_update   conservative update, one thread per cell
//   k_adv_pwchi    rhoX update of advect_rk's y sweep
//   k_adv_mass     face mass fluxes rhoY u / rhoY v, one thread per inner face
// The sweeps are bandwidth-trivial next to the projection's solve; no sweep
// reads what its own launch writes (faces read cells, updates read faces).
#include "bella_advect.cuh"
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
    const int ns = adv_ns(G, 1);
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)adv_nl(G, 1) * ns) return;
    const int l = (int)(e / ns), c = (int)(e - (long long)l * ns);
    pw[adv_cell(G, 1, l, c)] = lmbda * (fy.f[5][adv_face(G, 1, l, c)] - fy.f[5][adv_face(G, 1, l, c + 1)]);
}

__global__ void k_adv_mass(AdvGeom G, int s, AdvFields F, double *mflux) {
    const int nf = adv_ns(G, s) - 1;                          // inner faces 1 .. ns-1 of an inner line
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)adv_nl(G, s) * nf) return;
    const int l = (int)(e / nf), f = 1 + (int)(e - (long long)l * nf);
    if (adv_inner_line(G, s, l)) mflux[adv_face(G, s, l, f)] = adv_mass(G, s, l, f, F);
}

namespace {

int blocks(long long n) { return (int)((n + 255) / 256); }

struct DevEx {
    AdvGeom G;
    AdvFields F;
    AdvFaces fl[3];
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
    void mass() {
        for (int s = 0; s < G.nd; ++s)
            k_adv_mass<<<blocks((long long)adv_nl(G, s) * (adv_ns(G, s) - 1)), 256, 0, st>>>(G, s, F, fl[s].f[4]);
    }
    void pwchi(double lmbda) {
        if (!pw) return;
        k_adv_pwchi<<<blocks((long long)adv_nl(G, 1) * adv_ns(G, 1)), 256, 0, st>>>(G, fl[1], lmbda, pw);
    }
};

bool adv_setup(const bella_adv2d *a, DevEx &ex, void *stream) {
    if (!a || a->inx < 5 || a->iny < 5) return false;
    const double *req[] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0, a->strat_inv};
    for (const double *p : req)
        if (!p) return false;
    for (int q = 0; q < 6; ++q)
        if (!a->fx[q] || !a->fy[q]) return false;
    AdvGeom &G = ex.G;
    G.nd = 2;
    G.ic[0] = a->inx + 3; G.ic[1] = a->iny + 3; G.ic[2] = 1;
    G.bc[0] = a->x_wall ? 1 : 0; G.bc[1] = a->y_wall ? 1 : 0; G.bc[2] = 0;
    G.d[0] = a->dx; G.d[1] = a->dy; G.d[2] = 1.0;
    G.g = a->g; G.gamm = a->gamm; G.is_compressible = a->is_compressible;
    double *f[6] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX};
    for (int q = 0; q < 6; ++q) {
        ex.F.f[q] = f[q];
        ex.fl[0].f[q] = a->fx[q];
        ex.fl[1].f[q] = a->fy[q];
        ex.fl[2].f[q] = nullptr;
    }
    ex.rhoY0 = a->hydro_rhoY0; ex.strat_inv = a->strat_inv; ex.pw = a->pwchi;
    ex.st = (cudaStream_t)stream;
    return true;
}

bool adv_setup(const bella_adv3d *a, DevEx &ex, void *stream) {
    if (!a || a->inx < 5 || a->iny < 5 || a->inz < 5) return false;
    const double *req[] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0, a->strat_inv};
    for (const double *p : req)
        if (!p) return false;
    for (int q = 0; q < 6; ++q)
        if (!a->fx[q] || !a->fy[q] || !a->fz[q]) return false;
    AdvGeom &G = ex.G;
    G.nd = 3;
    G.ic[0] = a->inx + 3; G.ic[1] = a->iny + 3; G.ic[2] = a->inz + 3;
    G.bc[0] = a->x_wall ? 1 : 0; G.bc[1] = a->y_wall ? 1 : 0; G.bc[2] = a->z_wall ? 1 : 0;
    G.d[0] = a->dx; G.d[1] = a->dy; G.d[2] = a->dz;
    G.g = a->g; G.gamm = a->gamm; G.is_compressible = a->is_compressible;
    double *f[6] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX};
    for (int q = 0; q < 6; ++q) {
        ex.F.f[q] = f[q];
        ex.fl[0].f[q] = a->fx[q];
        ex.fl[1].f[q] = a->fy[q];
        ex.fl[2].f[q] = a->fz[q];
    }
    ex.rhoY0 = a->hydro_rhoY0; ex.strat_inv = a->strat_inv; ex.pw = a->pwchi;
    ex.st = (cudaStream_t)stream;
    return true;
}

}  // namespace
}  // namespace bella

using namespace bella;

template <class A>
static int fluxes_impl(const A *a, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    ex.mass();
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

template <class A>
static int advect_impl(const A *a, double dt, int odd, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    adv_strang(ex, ex.G, dt, odd);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

template <class A>
static int advect_rk_impl(const A *a, double dt, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    adv_rk(ex, ex.G, dt);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// set_explicit_boundary_data (boundary.py:7-216) of the whole state: axis by axis
template <class A>
static int boundary_impl(const A *a, void *stream) {
    DevEx ex;
    if (!adv_setup(a, ex, stream)) return BELLA_EINVAL;
    for (int s = 0; s < ex.G.nd; ++s) ex.bd(s);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" {
int bella_advective_fluxes2d(const bella_adv2d *a, void *stream) { return fluxes_impl(a, stream); }
int bella_advect2d(const bella_adv2d *a, double dt, int odd, void *stream) { return advect_impl(a, dt, odd, stream); }
int bella_advect_rk2d(const bella_adv2d *a, double dt, void *stream) { return advect_rk_impl(a, dt, stream); }
int bella_boundary2d(const bella_adv2d *a, void *stream) { return boundary_impl(a, stream); }
int bella_advective_fluxes3d(const bella_adv3d *a, void *stream) { return fluxes_impl(a, stream); }
int bella_advect3d(const bella_adv3d *a, double dt, int odd, void *stream) { return advect_impl(a, dt, odd, stream); }
int bella_advect_rk3d(const bella_adv3d *a, double dt, void *stream) { return advect_rk_impl(a, dt, stream); }
int bella_boundary3d(const bella_adv3d *a, void *stream) { return boundary_impl(a, stream); }
}
