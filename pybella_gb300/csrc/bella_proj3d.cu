// bella_proj3d.cu -- the 3D implicit nodal projection on the device.
//
// The reference's projection pieces are dimension-generic and run in 3D; its
// step (second_projection.py:97-277) cannot (the 3D branch uses diag_inv and p2
// before assignment, :183-203).  bella_projection3d assembles the step from the
// 3D pieces with the glue of the reference's 2D branch: unknowns are the inner
// nodes, hplus the cells around them, hcenter and diag_inv (the 3D
// precon_diag_prepare) at those nodes, the right-hand side the node.isc
// divergence scaled by 1/dt and diag_inv, vector order C over (x, y, z)
// (second_projection.py:224), corrf = dt * coriolis_strength[0] (laplacian.py:894).
//
// Kernels (one thread per cell / node / line; bandwidth-trivial next to the solve):
//   k3_bd_axis        set_boundary along x or z: wrap / symmetric   boundary.py:135-216
//   k3_bd_grav        hydrostatic ghost planes along y (gravity)     boundary.py:56-132, :248-281
//   k3_coeff_cells    wplus (all three axes) -> packed cell plane    second_projection.py:308-341
//   k3_coeff_nodes    wcenter, wall scaling, regime, 3D diagonal     :343-356, :147-153, laplacian.py:1284-1356
//   k3_zero_ghost     y-wall ghost momenta of divergence_nodes       :542-551
//   k3_divergence     divergence_nodes (3D branch), /dt, *diag_inv   :556-570, :139, :170
//   k3_ghost          set_ghostnodes_p2 along one axis               boundary.py:296-369
//   k3_correction     grad_nodes + correction_nodes (3D)             :280-306, :496-521, :604-646
//   k3_scatter, k3_add   p2_full[i2] = x; p2_nodes += p2_full        :265-275
// Array layout: the reference's NumPy C order over (x, y, z), ghosts included.
#include <cstring>

#include "bella_internal.cuh"

namespace bella {

struct Proj3Dev {
    int icx, icy, icz;     // cells incl. ghosts (inx+3, iny+3, inz+3)
    int ncx, ncy, ncz;     // nodes incl. ghosts (inx+4, iny+4, inz+4)
    int bc[3];             // 0 periodic, 1 wall
    double dx, dy, dz, dt, Msq, g, gamm, nonhydro, compressibility, wh1, wv, wh2;
    double xsign;          // divergence x term: -1 as divergence_nodes' 3D branch, +1 as its 2D branch
    int is_compressible;
};

__device__ __forceinline__ long long c3(const Proj3Dev &P, int i, int j, int k) {
    return ((long long)i * P.icy + j) * P.icz + k;
}
__device__ __forceinline__ long long n3(const Proj3Dev &P, int i, int j, int k) {
    return ((long long)i * P.ncy + j) * P.ncz + k;
}

// set_boundary along axis dim (0: x, 1: y without gravity, 2: z): one thread per
// line of cells along dim.  Periodic: np.pad(inner, 'wrap'); wall: 'symmetric' for
// rho, rhou, rhoY, rhoX, negative-symmetric for rhov, rhow left as it is
// (boundary.py:156-166).
__global__ void k3_bd_axis(Proj3Dev P, int dim, double *f0, double *f1, double *f2, double *f3, double *f4,
                           double *f5) {
    const int ext[3] = {P.icx, P.icy, P.icz};
    const int da = dim == 0 ? 1 : 0, db = dim == 2 ? 1 : 2;     // the other two axes
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)ext[da] * ext[db]) return;
    int c[3];
    c[da] = (int)(e / ext[db]);
    c[db] = (int)(e - (long long)c[da] * ext[db]);
    const int n = ext[dim];
    auto at = [&](double *a, int t) -> double & {
        c[dim] = t;
        return a[c3(P, c[0], c[1], c[2])];
    };
    double *F[6] = {f0, f1, f2, f3, f4, f5};                   // rho, rhou, rhov, rhow, rhoY, rhoX
    for (int q = 0; q < 6; ++q) {
        double *a = F[q];
        if (P.bc[dim] == 0) {
            at(a, 0) = at(a, n - 4);
            at(a, 1) = at(a, n - 3);
            at(a, n - 2) = at(a, 2);
            at(a, n - 1) = at(a, 3);
        } else {
            if (q == 3) continue;
            const double sg = (q == 2) ? -1.0 : 1.0;
            at(a, 1) = sg * at(a, 2);
            at(a, 0) = sg * at(a, 3);
            at(a, n - 2) = sg * at(a, n - 3);
            at(a, n - 1) = sg * at(a, n - 4);
        }
    }
}

// hydrostatic reflection along y (boundary.py:56-132, non-Lamb branch), one thread per (x, z) column
__global__ void k3_bd_grav(Proj3Dev P, double *rho, double *rhou, double *rhov, double *rhow, double *rhoY,
                           double *rhoX, const double *hydro_rhoY0, const double *strat_inv) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icz) return;
    const int i = (int)(e / P.icz), k = (int)(e - (long long)i * P.icz);
    const int n = P.icy;
    const double gamm = P.gamm, gm1 = gamm - 1.0, gm1inv = 1.0 / gm1, Gamma = gm1 / gamm;
    const int igy = 2;
    double direction = -1.0;
    int offset = 0;
    for (int side = 0; side < 2; ++side) {
        direction *= -1.0;
        for (int cur = igy - 1; cur >= 0; --cur) {      // get_gravity_padding (boundary.py:248-281)
            const int cur_idx = cur + offset * ((n - 1) - 2 * cur);
            const long long L = c3(P, i, (int)(cur_idx + direction), k);
            const long long S_ = c3(P, i, (int)(offset * n + direction * (2 * igy - (1 - offset) - cur)), k);
            const long long I = c3(P, i, cur_idx, k);
            const double Y_last = rhoY[L] / rho[L];
            const double rhoYv_image = -rhov[S_] * rhoY[S_] / rho[S_];
            const double S = strat_inv[cur_idx];
            const double dpi = direction * (Gamma * P.g) * 0.5 * P.dy * (1.0 / Y_last + S);
            const double rY = (P.is_compressible == 1) ? pow(pow(rhoY[L], gm1) + dpi, gm1inv) : hydro_rhoY0[cur_idx];
            const double r = rY * S;
            const double v = rhoYv_image / rY;
            const double u = rhou[S_] / rho[S_];
            const double w = rhow[S_] / rho[S_];
            const double X = rhoX[S_] / rho[S_];
            rho[I] = r;
            rhou[I] = r * u * 1.0;
            rhov[I] = r * v;
            rhow[I] = r * w * 1.0;
            rhoY[I] = rY;
            rhoX[I] = r * X;
        }
        offset += 1;
    }
}

// dS/dy on cell plane j from the node background S0 (variable.py:162-177)
__device__ __forceinline__ double dSdy3(const Proj3Dev &P, const double *S0n, int j) {
    return (S0n[j + 1] - S0n[j]) / P.dy;
}

// wplus = Gammainv * rhoY * Y of the coefficient state on every cell, and the
// cells around the inner nodes packed (inx+1)(iny+1)(inz+1) for the operator
// (the same plane serves hplusx, hplusy, hplusz); rhoY^(2-gamma) per cell for
// wcenter, so that each node sums eight values instead of taking eight pows
__global__ void k3_coeff_cells(Proj3Dev P, const double *rhoC, const double *rhoYC, double *wplus0, double *hpk,
                               double *pwc) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy * P.icz) return;
    const int i = (int)(e / ((long long)P.icy * P.icz));
    const int r = (int)(e - (long long)i * P.icy * P.icz);
    const int j = r / P.icz, k = r - j * P.icz;
    const double Gammainv = P.gamm / (P.gamm - 1.0);
    const double Y = rhoYC[e] / rhoC[e];
    const double w = Gammainv * rhoYC[e] * Y;
    wplus0[e] = w;
    pwc[e] = pow(rhoYC[e], 2.0 - P.gamm);
    if (i >= 1 && i <= P.icx - 2 && j >= 1 && j <= P.icy - 2 && k >= 1 && k <= P.icz - 2)
        hpk[((long long)(i - 1) * (P.icy - 2) + (j - 1)) * (P.icz - 2) + (k - 1)] = w;
}

// node.isc: wcenter = ccenter * box(rhoY^(2-gamma)) / 8, halved on wall rows,
// times compressibility in the pseudo-incompressible regime; the 3D Jacobi
// diagonal (laplacian.py:1334-1356: coefficient 0.0625, the x-y cross terms
// kept as the reference has them); inner nodes packed -> hc, dinv
__global__ void k3_coeff_nodes(Proj3Dev P, const double *pwc, const double *wplus0, double *dinv_isc, double *hc,
                               double *dinv) {
    const int nix = P.icx - 1, niy = P.icy - 1, niz = P.icz - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy * niz) return;
    const int a = (int)(e / ((long long)niy * niz));
    const int r = (int)(e - (long long)a * niy * niz);
    const int b = r / niz, c = r - b * niz;
    const double gm1inv = 1.0 / (P.gamm - 1.0);
    const double ccenter = -P.Msq * gm1inv / (P.dt * P.dt);
    double s = 0.0, S = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const long long cc = c3(P, a + (q >> 2), b + ((q >> 1) & 1), c + (q & 1));
        s += pwc[cc];
        S += wplus0[cc];
    }
    double wc = ccenter * s / 8.0;
    {
        const int cd[3] = {a, b, c}, n[3] = {nix, niy, niz};
        wc *= wall_scale(3, cd, n, P.bc, 0.5);
    }
    if (P.is_compressible != 1) wc *= P.compressibility;        // second_projection.py:147-153
    const double cf = 0.0625;
    const double wxx = cf / (P.dx * P.dx), wyy = cf / (P.dy * P.dy), wzz = cf / (P.dz * P.dz);
    const double wxy = cf / (P.dx * P.dy), wyx = cf / (P.dy * P.dx);
    double diag = -wxx * S;
    diag -= wyy * S;
    diag -= wxy * S;
    diag -= wyx * S;
    diag -= wzz * S;
    diag += wc;
    const double di = 1.0 / diag;
    dinv_isc[e] = di;
    if (a >= 1 && a <= nix - 2 && b >= 1 && b <= niy - 2 && c >= 1 && c <= niz - 2) {
        const long long pk = ((long long)(a - 1) * (niy - 2) + (b - 1)) * (niz - 2) + (c - 1);
        hc[pk] = wc;
        dinv[pk] = di;
    }
}

// divergence_nodes at a y wall: momenta of the two ghost planes on each side zeroed
__global__ void k3_zero_ghost(Proj3Dev P, double *rhou, double *rhov, double *rhow) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icz || P.bc[1] != 1) return;
    const int i = (int)(e / P.icz), k = (int)(e - (long long)i * P.icz);
    const int n = P.icy;
    const int rows[4] = {0, 1, n - 2, n - 1};
    for (int t = 0; t < 4; ++t) {
        const long long q = c3(P, i, rows[t], k);
        rhou[q] = 0.0;
        rhov[q] = 0.0;
        rhow[q] = 0.0;
    }
}

// Y = rhoY / rho per cell for the divergence (eight cells share it per node)
__global__ void k3_cell_y(Proj3Dev P, const double *rho, const double *rhoY, double *Yc) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e < (long long)P.icx * P.icy * P.icz) Yc[e] = rhoY[e] / rho[e];
}

// divergence_nodes, 3D branch (second_projection.py:556-570) on node.isc, with the
// reference's sign on the x term (Ux = -0.5 * (...), :563) or the 2D branch's
// (P.xsign); /dt (:139), the
// regime mix (:149-150), b = (rhs * diag_inv)[inner] in C order (:170, :224)
__global__ void k3_divergence(Proj3Dev P, const double *Yc, const double *rhou, const double *rhov,
                              const double *rhow, const double *dinv_isc, double *rhs_isc, double *bvec) {
    const int nix = P.icx - 1, niy = P.icy - 1, niz = P.icz - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy * niz) return;
    const int a = (int)(e / ((long long)niy * niz));
    const int r = (int)(e - (long long)a * niy * niz);
    const int b = r / niz, c = r - b * niz;
    auto Y = [&](int i, int j, int k) { return Yc[c3(P, i, j, k)]; };
    auto qu = [&](int i, int j, int k) { return rhou[c3(P, i, j, k)] * Y(i, j, k); };
    auto qv = [&](int i, int j, int k) { return rhov[c3(P, i, j, k)] * Y(i, j, k); };
    auto qw = [&](int i, int j, int k) { return rhow[c3(P, i, j, k)] * Y(i, j, k); };
    double ux[2], vy[2], wz[2];
    for (int t = 0; t < 2; ++t) {
        const double d0 = (qu(a + 1, b, c + t) - qu(a, b, c + t)) / P.dx;
        const double d1 = (qu(a + 1, b + 1, c + t) - qu(a, b + 1, c + t)) / P.dx;
        ux[t] = 0.5 * (d0 + d1);
        const double e0 = (qv(a, b + 1, c + t) - qv(a, b, c + t)) / P.dy;
        const double e1 = (qv(a + 1, b + 1, c + t) - qv(a + 1, b, c + t)) / P.dy;
        vy[t] = 0.5 * (e0 + e1);
        const double f0 = (qw(a, b + t, c + 1) - qw(a, b + t, c)) / P.dz;
        const double f1 = (qw(a + 1, b + t, c + 1) - qw(a + 1, b + t, c)) / P.dz;
        wz[t] = 0.5 * (f0 + f1);
    }
    const double Ux = (0.5 * P.xsign) * (ux[0] + ux[1]);
    const double Vy = 0.5 * (vy[0] + vy[1]);
    const double Wz = 0.5 * (wz[0] + wz[1]);
    double rhs = (Ux + Vy + Wz) / P.dt;
    if (P.is_compressible == 0) rhs = P.compressibility * rhs + (1.0 - P.compressibility) * rhs;
    rhs_isc[e] = rhs;
    if (a >= 1 && a <= nix - 2 && b >= 1 && b <= niy - 2 && c >= 1 && c <= niz - 2)
        bvec[((long long)(a - 1) * (niy - 2) + (b - 1)) * (niz - 2) + (c - 1)] = rhs * dinv_isc[e];
}

// set_ghostnodes_p2 along axis dim: periodic_plus_one (boundary.py:348-369) or
// 'reflect', one thread per line of nodes along dim
__global__ void k3_ghost(Proj3Dev P, int dim, double *p) {
    const int ext[3] = {P.ncx, P.ncy, P.ncz};
    const int da = dim == 0 ? 1 : 0, db = dim == 2 ? 1 : 2;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)ext[da] * ext[db]) return;
    int c[3];
    c[da] = (int)(e / ext[db]);
    c[db] = (int)(e - (long long)c[da] * ext[db]);
    const int n = ext[dim];
    auto at = [&](int t) -> double & {
        c[dim] = t;
        return p[n3(P, c[0], c[1], c[2])];
    };
    if (P.bc[dim] == 0) {
        const double h0 = at(n - 5), h1 = at(n - 4), h2 = at(n - 3);
        const double t0 = at(2), t1 = at(3), t2 = at(4);
        at(0) = h0; at(1) = h1; at(2) = h2;
        at(n - 3) = t0; at(n - 2) = t1; at(n - 1) = t2;
    } else {
        at(0) = at(4);
        at(1) = at(3);
        at(n - 2) = at(n - 4);
        at(n - 1) = at(n - 5);
    }
}

// correction_nodes (second_projection.py:280-306) with the 3D grad_nodes (:496-521:
// corners in itertools.product order, signs as the reference lists them) and the
// Coriolis inverse (:604-646), on every cell
__global__ void k3_correction(Proj3Dev P, const double *p, const double *rho, double *rhou, double *rhov,
                              double *rhow, const double *rhoY, double *rhoX, const double *S0n, double updt_chi) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy * P.icz) return;
    const int i = (int)(e / ((long long)P.icy * P.icz));
    const int r = (int)(e - (long long)i * P.icy * P.icz);
    const int j = r / P.icz, k = r - j * P.icz;
    double Dpx = 0.0, Dpy = 0.0, Dpz = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int ox = q >> 2, oy = (q >> 1) & 1, oz = q & 1;
        const double v = p[n3(P, i + ox, j + oy, k + oz)];
        Dpx = Dpx + (ox ? 1.0 : -1.0) * v;
        Dpy = Dpy + (oy ? 1.0 : -1.0) * v;
        Dpz = Dpz + (oz ? 1.0 : -1.0) * v;
    }
    Dpx = Dpx * (0.25 / P.dx);
    Dpy = Dpy * (0.25 / P.dy);
    Dpz = Dpz * (0.25 / P.dz);
    const double Gammainv = P.gamm / (P.gamm - 1.0);
    const double thinv = rho[e] / rhoY[e];
    const double Y = rhoY[e] / rho[e];
    const double coeff = Gammainv * rhoY[e] * Y;
    const double U0 = -P.dt * coeff * Dpx, V0 = -P.dt * coeff * Dpy, W0 = -P.dt * coeff * Dpz;
    const double ds = dSdy3(P, S0n, j);
    const CorCoef cf = cor_coef(P, Y, ds);
    const double U = cf.denom * (cf.uu * U0 + cf.uv * V0 + cf.uw * W0);
    const double V = cf.denom * (cf.vu * U0 + cf.vv * V0 + cf.vw * W0);
    const double W = cf.denom * (cf.wu * U0 + cf.wv * V0 + cf.ww * W0);
    rhou[e] = rhou[e] + thinv * U;
    const double rv = rhov[e] + thinv * V;
    rhov[e] = rv;
    rhow[e] = rhow[e] + thinv * W;
    rhoX[e] = rhoX[e] + (-updt_chi * P.dt * ds * rv);
}

// p2_full = 0; p2_full[2:-2, 2:-2, 2:-2] = x.reshape(inx, iny, inz)
__global__ void k3_scatter(Proj3Dev P, const double *x, double *pfull) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.ncx * P.ncy * P.ncz) return;
    const int i = (int)(e / ((long long)P.ncy * P.ncz));
    const int r = (int)(e - (long long)i * P.ncy * P.ncz);
    const int j = r / P.ncz, k = r - j * P.ncz;
    const int inx = P.ncx - 4, iny = P.ncy - 4, inz = P.ncz - 4;
    double v = 0.0;
    if (i >= 2 && i < 2 + inx && j >= 2 && j < 2 + iny && k >= 2 && k < 2 + inz)
        v = x[((long long)(i - 2) * iny + (j - 2)) * inz + (k - 2)];
    pfull[e] = v;
}

__global__ void k3_add(long long n, double *a, const double *b) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e < n) a[e] += b[e];
}

}  // namespace bella

using namespace bella;

static int grid3(long long n) { return (int)((n + 255) / 256); }

static void bd3(const Proj3Dev &P, double *const F[6], const double *rhoY0, const double *strat_inv,
                cudaStream_t s, long long &launches) {
    const long long lx = (long long)P.icy * P.icz, ly = (long long)P.icx * P.icz, lz = (long long)P.icx * P.icy;
    k3_bd_axis<<<grid3(lx), 256, 0, s>>>(P, 0, F[0], F[1], F[2], F[3], F[4], F[5]);
    if (P.g != 0.0)
        k3_bd_grav<<<grid3(ly), 256, 0, s>>>(P, F[0], F[1], F[2], F[3], F[4], F[5], rhoY0, strat_inv);
    else
        k3_bd_axis<<<grid3(ly), 256, 0, s>>>(P, 1, F[0], F[1], F[2], F[3], F[4], F[5]);
    k3_bd_axis<<<grid3(lz), 256, 0, s>>>(P, 2, F[0], F[1], F[2], F[3], F[4], F[5]);
    launches += 3;
}

static void ghost3(const Proj3Dev &P, double *p, cudaStream_t s, long long &launches) {
    k3_ghost<<<grid3((long long)P.ncy * P.ncz), 256, 0, s>>>(P, 0, p);
    k3_ghost<<<grid3((long long)P.ncx * P.ncz), 256, 0, s>>>(P, 1, p);
    k3_ghost<<<grid3((long long)P.ncx * P.ncy), 256, 0, s>>>(P, 2, p);
    launches += 3;
}

extern "C" int bella_projection3d(bella_ws *ws, const bella_proj3d *a, const bella_solve_opts *opts,
                                  bella_solve_stats *stats, void *stream) {
    if (!ws || !a) return BELLA_EINVAL;
    if (a->inx < 5 || a->iny < 5 || a->inz < 5 || !a->rho || !a->rhou || !a->rhov || !a->rhow || !a->rhoY ||
        !a->rhoX || !a->p2 || !a->hydro_rhoY0 || !a->S0n || !a->strat_inv)
        return BELLA_EINVAL;
    if (a->precond != 0 && (a->precond != 1 || !a->y_wall)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    Proj3Dev P;
    P.icx = a->inx + 3; P.icy = a->iny + 3; P.icz = a->inz + 3;
    P.ncx = a->inx + 4; P.ncy = a->iny + 4; P.ncz = a->inz + 4;
    P.bc[0] = a->x_wall ? 1 : 0; P.bc[1] = a->y_wall ? 1 : 0; P.bc[2] = a->z_wall ? 1 : 0;
    P.dx = a->dx; P.dy = a->dy; P.dz = a->dz; P.dt = a->dt; P.Msq = a->Msq; P.g = a->g; P.gamm = a->gamm;
    P.nonhydro = a->nonhydro; P.compressibility = a->compressibility;
    P.wh1 = a->dt * a->coriolis[0]; P.wv = a->dt * a->coriolis[1]; P.wh2 = a->dt * a->coriolis[2];
    P.is_compressible = a->is_compressible;
    P.xsign = a->div_sign_2d ? 1.0 : -1.0;
    const long long ncell = (long long)P.icx * P.icy * P.icz, nnode = (long long)P.ncx * P.ncy * P.ncz;
    const long long nisc = (long long)(P.icx - 1) * (P.icy - 1) * (P.icz - 1);
    const long long nin = (long long)a->inx * a->iny * a->inz;
    const long long npk = (long long)(a->inx + 1) * (a->iny + 1) * (a->inz + 1);
    // scratch: wplus0, dinv_isc, rhs_isc, packed cells, hc, dinv, b, x, pfull, a cell field
    // (rhoY^(2-gamma) for the coefficients, then Y for the divergence)
    const size_t need = (size_t)(2 * ncell + 2 * nisc + npk + 4 * nin + nnode);
    if (ws->proj_cap < need) {
        cudaFree(ws->proj_buf);
        ws->proj_buf = nullptr;
        ws->proj_cap = 0;
        if (cudaMalloc(&ws->proj_buf, need * sizeof(double)) != cudaSuccess) return BELLA_ECUDA;
        ws->proj_cap = need;
    }
    double *q = ws->proj_buf;
    double *wplus0 = q; q += ncell;
    double *dinv_isc = q; q += nisc;
    double *rhs_isc = q; q += nisc;
    double *hpk = q; q += npk;
    double *hc = q; q += nin;
    double *dinv = q; q += nin;
    double *bvec = q; q += nin;
    double *xvec = q; q += nin;
    double *pfull = q; q += nnode;
    double *cellf = q;

    const bool has0 = a->rho0 != nullptr;
    double *const F[6] = {a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX};
    double *const C[6] = {has0 ? a->rho0 : a->rho, has0 ? a->rhou0 : a->rhou, has0 ? a->rhov0 : a->rhov,
                          has0 ? a->rhow0 : a->rhow, has0 ? a->rhoY0 : a->rhoY, has0 ? a->rhoX0 : a->rhoX};
    long long L = 0;
    // 1. coefficient state: boundary data of Sol0 or Sol (second_projection.py:113-118)
    bd3(P, C, a->hydro_rhoY0, a->strat_inv, s, L);
    // 2. ghost nodes of p2, correction with the old p2, boundary data (:130-132)
    ghost3(P, a->p2, s, L);
    k3_correction<<<grid3(ncell), 256, 0, s>>>(P, a->p2, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX,
                                              a->S0n, 0.0);
    bd3(P, F, a->hydro_rhoY0, a->strat_inv, s, L);
    // 3. coefficients from the coefficient state and the diagonal
    k3_coeff_cells<<<grid3(ncell), 256, 0, s>>>(P, C[0], C[4], wplus0, hpk, cellf);
    k3_coeff_nodes<<<grid3(nisc), 256, 0, s>>>(P, cellf, wplus0, dinv_isc, hc, dinv);
    // 4. divergence right-hand side (:134-170, :224)
    k3_zero_ghost<<<grid3((long long)P.icx * P.icz), 256, 0, s>>>(P, a->rhou, a->rhov, a->rhow);
    k3_cell_y<<<grid3(ncell), 256, 0, s>>>(P, a->rho, a->rhoY, cellf);
    k3_divergence<<<grid3(nisc), 256, 0, s>>>(P, cellf, a->rhou, a->rhov, a->rhow, dinv_isc, rhs_isc, bvec);
    L += 6;
    if (a->rhs_out) cudaMemcpyAsync(a->rhs_out, rhs_isc, nisc * sizeof(double), cudaMemcpyDeviceToDevice, s);
    ws->launches += L;
    if (cudaGetLastError() != cudaSuccess) return BELLA_ECUDA;
    // 5. operator (the closure of stencil_27pt, laplacian.py:872-896) and solve (:230)
    const bool hc_on = !(a->is_compressible == 0 && a->compressibility == 0.0);
    bella_op3d op;
    op.nx = a->inx; op.ny = a->iny; op.nz = a->inz;
    op.x_wall = a->x_wall; op.y_wall = a->y_wall; op.z_wall = a->z_wall;
    op.dx = a->dx; op.dy = a->dy; op.dz = a->dz;
    op.corrf = a->dt * a->coriolis[0];
    op.hplusx = hpk; op.hplusy = hpk; op.hplusz = hpk;
    op.hcenter = hc_on ? hc : nullptr;
    op.diag_inv = dinv;
    int rc = bella_op3d_set(ws, &op, stream);
    if (rc != BELLA_OK) return rc;
    bella_solve_opts o;
    if (opts) o = *opts; else bella_solve_opts_default(&o);
    o.x0_zero = 1;
    int st;
    if (a->precond == 1) {
        // the workspace's background solve, re-derived from this call's coefficients
        // (made anew when the grid or a boundary kind changed)
        if (!ws->sp_cache || bella_spectral3d_update(ws->sp_cache, &op, stream) != BELLA_OK) {
            bella_spectral3d_destroy(ws->sp_cache);
            ws->sp_cache = nullptr;
            rc = bella_spectral3d_create(&ws->sp_cache, &op, ws->device, stream);
            if (rc != BELLA_OK) return rc;
        }
        st = bella_fbicgstab_pc(ws, ws->sp_cache, nullptr, 0, bvec, xvec, &o, stats, stream);
    } else {
        st = bella_bicgstab(ws, bvec, xvec, &o, stats, stream);
    }
    if (st < 0) return st;
    // 6. p2_full, ghost nodes, correction with updt_chi = 1, p2 += p2_full, ghosts, boundary data (:265-277)
    L = 0;
    k3_scatter<<<grid3(nnode), 256, 0, s>>>(P, xvec, pfull);
    ghost3(P, pfull, s, L);
    k3_correction<<<grid3(ncell), 256, 0, s>>>(P, pfull, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX,
                                              a->S0n, 1.0);
    k3_add<<<grid3(nnode), 256, 0, s>>>(nnode, a->p2, pfull);
    ghost3(P, a->p2, s, L);
    bd3(P, F, a->hydro_rhoY0, a->strat_inv, s, L);
    ws->launches += L + 3;
    if (cudaGetLastError() != cudaSuccess) return BELLA_ECUDA;
    return st;
}
