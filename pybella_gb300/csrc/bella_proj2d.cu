// bella_proj2d.cu -- the whole 2D implicit nodal projection on the device:
// euler_backward_non_advective_impl_part (second_projection.py:97-277).
//
// Kernels (one thread per cell / node / column; the arrays are small and
// the work is bandwidth-trivial next to the solve):
//   k_bd_x / k_bd_y     set_explicit_boundary_data   boundary.py:7-216
//   k_coeff_cells       operator_coefficients_nodes  second_projection.py:308-341
//                       + multiply_inverse_coriolis coefficients  :604-633,651
//   k_coeff_nodes       wcenter, wall scaling, Jacobi diagonal     :343-356, laplacian.py:1284-1356
//   k_divergence        divergence_nodes, /dt, *diag_inv, packing  :525-575, :134-170, :214
//   k_ghost_x / _y      set_ghostnodes_p2 (periodic_plus_one, reflect)  boundary.py:296-369
//   k_correction        grad_nodes + correction_nodes              :280-306, :496-521
//   k_scatter_add       p2_full[i2] = x; p2_nodes += p2_full       :241-245, :275
// and the explicit parts (bella_euler_forward2d, bella_expl_part2d):
//   k_fw_div / k_fw_cells / k_fw_nodes   euler_forward_non_advective  :22-74
//   k_ex_cells          euler_backward_non_advective_expl_part       :77-92
// Array layout is the reference's NumPy C order over (x, y).
#include <cstring>
#include <string>

#include <vector>

#include "bella_internal.cuh"

namespace bella {

struct ProjDev {
    int icx, icy;          // cells incl. ghosts (inx+3, iny+3)
    int ncx, ncy;          // nodes incl. ghosts (inx+4, iny+4)
    int xbc, ybc;          // 0 periodic, 1 wall
    double dx, dy, dt, Msq, g, gamm, nonhydro, compressibility, wh1, wv, wh2;
    int is_compressible;
};

__device__ __forceinline__ long long cidx(const ProjDev &P, int i, int j) { return (long long)i * P.icy + j; }
__device__ __forceinline__ long long nidx(const ProjDev &P, int i, int j) { return (long long)i * P.ncy + j; }

// ---- set_explicit_boundary_data, x direction (no gravity along x) -------------
// periodic: np.pad(..., 'wrap') of the inner cells; wall: 'symmetric' for
// rho, rhou, rhoY, rhoX, negative-symmetric for rhov, rhow left untouched
// (boundary.py:156-216).
__global__ void k_bd_x(ProjDev P, double *f0, double *f1, double *f2, double *f3, double *f4, double *f5) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P.icy) return;
    double *F[6] = {f0, f1, f2, f3, f4, f5};     // rho, rhou, rhov, rhow, rhoY, rhoX
    const int n = P.icx;
    for (int q = 0; q < 6; ++q) {
        double *a = F[q];
        if (P.xbc == 0) {
            a[cidx(P, 0, j)] = a[cidx(P, n - 4, j)];
            a[cidx(P, 1, j)] = a[cidx(P, n - 3, j)];
            a[cidx(P, n - 2, j)] = a[cidx(P, 2, j)];
            a[cidx(P, n - 1, j)] = a[cidx(P, 3, j)];
        } else {
            if (q == 3) continue;                         // rhow is not padded (boundary.py:161-166)
            const double sg = (q == 2) ? -1.0 : 1.0;
            a[cidx(P, 1, j)] = sg * a[cidx(P, 2, j)];
            a[cidx(P, 0, j)] = sg * a[cidx(P, 3, j)];
            a[cidx(P, n - 2, j)] = sg * a[cidx(P, n - 3, j)];
            a[cidx(P, n - 1, j)] = sg * a[cidx(P, n - 4, j)];
        }
    }
}

// ---- y direction: hydrostatic reflection along gravity (boundary.py:56-132)
// or wrap/symmetric when g == 0 -------------------------------------------------
__global__ void k_bd_y(ProjDev P, double *rho, double *rhou, double *rhov, double *rhow, double *rhoY,
                       double *rhoX, const double *hydro_rhoY0, const double *strat_inv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.icx) return;
    const int n = P.icy;
    if (P.g == 0.0) {
        double *F[6] = {rho, rhou, rhov, rhow, rhoY, rhoX};
        for (int q = 0; q < 6; ++q) {
            double *a = F[q];
            if (P.ybc == 0) {
                a[cidx(P, i, 0)] = a[cidx(P, i, n - 4)];
                a[cidx(P, i, 1)] = a[cidx(P, i, n - 3)];
                a[cidx(P, i, n - 2)] = a[cidx(P, i, 2)];
                a[cidx(P, i, n - 1)] = a[cidx(P, i, 3)];
            } else {
                if (q == 3) continue;
                const double sg = (q == 2) ? -1.0 : 1.0;
                a[cidx(P, i, 1)] = sg * a[cidx(P, i, 2)];
                a[cidx(P, i, 0)] = sg * a[cidx(P, i, 3)];
                a[cidx(P, i, n - 2)] = sg * a[cidx(P, i, n - 3)];
                a[cidx(P, i, n - 1)] = sg * a[cidx(P, i, n - 4)];
            }
        }
        return;
    }
    const double gamm = P.gamm, gm1 = gamm - 1.0, gm1inv = 1.0 / gm1, Gamma = gm1 / gamm;
    const int igy = 2;
    double direction = -1.0;
    int offset = 0;
    for (int side = 0; side < 2; ++side) {
        direction *= -1.0;
        for (int cur = igy - 1; cur >= 0; --cur) {      // get_gravity_padding (boundary.py:248-281)
            const int cur_idx = cur + offset * ((n - 1) - 2 * cur);
            const int nlast = (int)(cur_idx + direction);
            const int nsource = (int)(offset * n + direction * (2 * igy - (1 - offset) - cur));
            const int nimage = cur_idx;
            const double Y_last = rhoY[cidx(P, i, nlast)] / rho[cidx(P, i, nlast)];
            const double rhoYv_image = -rhov[cidx(P, i, nsource)] * rhoY[cidx(P, i, nsource)] / rho[cidx(P, i, nsource)];
            const double S = strat_inv[nimage];
            const double dpi = direction * (Gamma * P.g) * 0.5 * P.dy * (1.0 / Y_last + S);
            const double rY = (P.is_compressible == 1) ? pow(pow(rhoY[cidx(P, i, nlast)], gm1) + dpi, gm1inv)
                                                       : hydro_rhoY0[nimage];
            const double r = rY * S;
            const double v = rhoYv_image / rY;
            const double u = rhou[cidx(P, i, nsource)] / rho[cidx(P, i, nsource)];
            const double w = rhow[cidx(P, i, nsource)] / rho[cidx(P, i, nsource)];
            const double X = rhoX[cidx(P, i, nsource)] / rho[cidx(P, i, nsource)];
            rho[cidx(P, i, nimage)] = r;
            rhou[cidx(P, i, nimage)] = r * u * 1.0;
            rhov[cidx(P, i, nimage)] = r * v;
            rhow[cidx(P, i, nimage)] = r * w * 1.0;
            rhoY[cidx(P, i, nimage)] = rY;
            rhoX[cidx(P, i, nimage)] = r * X;
        }
        offset += 1;
    }
}

// dS/dy on cell row j from the node background S0 (variable.py:162-177)
__device__ __forceinline__ double dSdy(const ProjDev &P, const double *S0n, int j) {
    return (S0n[j + 1] - S0n[j]) / P.dy;
}

// wplus (from the coefficient state) and the packed Coriolis planes (from Sol),
// written straight into the reference's packed operand layout:
//   packed cell (row cj, col ci) = cell (ci+1, cj+1), row stride inx+1
__global__ void k_coeff_cells(ProjDev P, const double *rhoC, const double *rhoYC, const double *rho,
                              const double *rhoY, const double *S0n, double *wplus0, double *hx, double *hy,
                              double *cxx, double *cyy, double *cxy, double *cyx) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy) return;
    const int i = (int)(e / P.icy), j = (int)(e - (long long)i * P.icy);
    const double Gammainv = P.gamm / (P.gamm - 1.0);
    const double Yc = rhoYC[e] / rhoC[e];
    const double w = Gammainv * rhoYC[e] * Yc;                   // second_projection.py:326-341
    wplus0[e] = w;
    if (i >= 1 && i <= P.icx - 2 && j >= 1 && j <= P.icy - 2) {
        const int nxp = P.icx - 2;                                // packed row stride = inx + 1
        const long long pk = (long long)(j - 1) * nxp + (i - 1);
        hx[pk] = w;
        hy[pk] = w;
        const double Y = rhoY[e] / rho[e];
        const CorCoef c = cor_coef(P, Y, dSdy(P, S0n, j));
        cxx[pk] = c.uu * c.denom;                                 // second_projection.py:651
        cyy[pk] = c.vv * c.denom;
        cxy[pk] = c.uv * c.denom;
        cyx[pk] = c.vu * c.denom;
    }
}

// node.isc quantities: wcenter (box of rhoY^(2-gamma)), wall scaling, the
// regime factor and the Jacobi diagonal; packed inner nodes -> hc, dinv.
__global__ void k_coeff_nodes(ProjDev P, const double *rhoYC, const double *wplus0, double *dinv_isc,
                              double *hc, double *dinv) {
    const int nix = P.icx - 1, niy = P.icy - 1;                   // node.isc
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy) return;
    const int a = (int)(e / niy), b = (int)(e - (long long)a * niy);
    const double gm1inv = 1.0 / (P.gamm - 1.0), cexp = 2.0 - P.gamm;
    const double ccenter = -P.Msq * gm1inv / (P.dt * P.dt);
    const double s = pow(rhoYC[cidx(P, a, b)], cexp) + pow(rhoYC[cidx(P, a + 1, b)], cexp) +
                     pow(rhoYC[cidx(P, a, b + 1)], cexp) + pow(rhoYC[cidx(P, a + 1, b + 1)], cexp);
    double wc = ccenter * s / 4.0;
    // scale_wall_node_values(wcenter, 0.5) on the node rows next to a wall (second_projection.py:356)
    {
        const int c[2] = {a, b}, n[2] = {nix, niy}, wall[2] = {P.xbc, P.ybc};
        wc *= wall_scale(2, c, n, wall, 0.5);
    }
    if (P.is_compressible != 1) wc *= P.compressibility;          // :147-153
    const double S = wplus0[cidx(P, a, b)] + wplus0[cidx(P, a + 1, b)] + wplus0[cidx(P, a, b + 1)] +
                     wplus0[cidx(P, a + 1, b + 1)];
    const double cf = 1.0 - 0.5 * 0.5;                            // laplacian.py:1318-1321
    const double wxx = cf / (P.dx * P.dx), wyy = cf / (P.dy * P.dy), wxy = cf / (P.dx * P.dy);
    double diag = -wxx * S;
    diag = diag - wyy * S;
    diag = diag - wxy * S;
    diag = diag - wxy * S;
    diag = diag + wc;
    const double di = 1.0 / diag;
    dinv_isc[e] = di;
    if (a >= 1 && a <= nix - 2 && b >= 1 && b <= niy - 2) {
        const int inx = nix - 2;
        const long long pk = (long long)(b - 1) * inx + (a - 1);
        hc[pk] = wc;
        dinv[pk] = di;
    }
}

// divergence_nodes: zero the y-ghost momenta at a wall (second_projection.py:542-551)
__global__ void k_zero_ghost_momenta(ProjDev P, double *rhou, double *rhov, double *rhow) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.icx || P.ybc != 1) return;
    const int n = P.icy;
    const int rows[4] = {0, 1, n - 2, n - 1};
    for (int r = 0; r < 4; ++r) {
        rhou[cidx(P, i, rows[r])] = 0.0;
        rhov[cidx(P, i, rows[r])] = 0.0;
        rhow[cidx(P, i, rows[r])] = 0.0;
    }
}

// rhs = (Ux + Vy) / dt on node.isc; b = (rhs * diag_inv)[1:-1,1:-1].T (second_projection.py:556-572, :139, :170, :214)
__global__ void k_divergence(ProjDev P, const double *rho, const double *rhou, const double *rhov,
                             const double *rhoY, const double *dinv_isc, double *rhs_isc, double *bvec) {
    const int nix = P.icx - 1, niy = P.icy - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy) return;
    const int a = (int)(e / niy), b = (int)(e - (long long)a * niy);
    auto qu = [&](int i, int j) { return rhou[cidx(P, i, j)] * (rhoY[cidx(P, i, j)] / rho[cidx(P, i, j)]); };
    auto qv = [&](int i, int j) { return rhov[cidx(P, i, j)] * (rhoY[cidx(P, i, j)] / rho[cidx(P, i, j)]); };
    const double d0 = (qu(a + 1, b) - qu(a, b)) / P.dx;
    const double d1 = (qu(a + 1, b + 1) - qu(a, b + 1)) / P.dx;
    const double Ux = 0.5 * (d0 + d1);
    const double e0 = (qv(a, b + 1) - qv(a, b)) / P.dy;
    const double e1 = (qv(a + 1, b + 1) - qv(a + 1, b)) / P.dy;
    const double Vy = 0.5 * (e0 + e1);
    double rhs = (Ux + Vy) / P.dt;
    if (P.is_compressible == 0) rhs = P.compressibility * rhs + (1.0 - P.compressibility) * rhs;   // :149-150
    rhs_isc[e] = rhs;
    if (a >= 1 && a <= nix - 2 && b >= 1 && b <= niy - 2) {
        const int inx = nix - 2;
        bvec[(long long)(b - 1) * inx + (a - 1)] = rhs * dinv_isc[e];
    }
}

// set_ghostnodes_p2 along x: periodic_plus_one (boundary.py:348-369) or reflect
__global__ void k_ghost_x(ProjDev P, double *p) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P.ncy) return;
    const int n = P.ncx;
    if (P.xbc == 0) {
        const double h0 = p[nidx(P, n - 5, j)], h1 = p[nidx(P, n - 4, j)], h2 = p[nidx(P, n - 3, j)];
        const double t0 = p[nidx(P, 2, j)], t1 = p[nidx(P, 3, j)], t2 = p[nidx(P, 4, j)];
        p[nidx(P, 0, j)] = h0; p[nidx(P, 1, j)] = h1; p[nidx(P, 2, j)] = h2;
        p[nidx(P, n - 3, j)] = t0; p[nidx(P, n - 2, j)] = t1; p[nidx(P, n - 1, j)] = t2;
    } else {
        p[nidx(P, 0, j)] = p[nidx(P, 4, j)];
        p[nidx(P, 1, j)] = p[nidx(P, 3, j)];
        p[nidx(P, n - 2, j)] = p[nidx(P, n - 4, j)];
        p[nidx(P, n - 1, j)] = p[nidx(P, n - 5, j)];
    }
}

__global__ void k_ghost_y(ProjDev P, double *p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.ncx) return;
    const int n = P.ncy;
    if (P.ybc == 0) {
        const double h0 = p[nidx(P, i, n - 5)], h1 = p[nidx(P, i, n - 4)], h2 = p[nidx(P, i, n - 3)];
        const double t0 = p[nidx(P, i, 2)], t1 = p[nidx(P, i, 3)], t2 = p[nidx(P, i, 4)];
        p[nidx(P, i, 0)] = h0; p[nidx(P, i, 1)] = h1; p[nidx(P, i, 2)] = h2;
        p[nidx(P, i, n - 3)] = t0; p[nidx(P, i, n - 2)] = t1; p[nidx(P, i, n - 1)] = t2;
    } else {
        p[nidx(P, i, 0)] = p[nidx(P, i, 4)];
        p[nidx(P, i, 1)] = p[nidx(P, i, 3)];
        p[nidx(P, i, n - 2)] = p[nidx(P, i, n - 4)];
        p[nidx(P, i, n - 1)] = p[nidx(P, i, n - 5)];
    }
}

// correction_nodes (second_projection.py:280-306) with grad_nodes (:496-521), on every cell
__global__ void k_correction(ProjDev P, const double *p, double *rho, double *rhou, double *rhov, double *rhow,
                             const double *rhoY, double *rhoX, const double *S0n, double updt_chi) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy) return;
    const int i = (int)(e / P.icy), j = (int)(e - (long long)i * P.icy);
    const double a00 = p[nidx(P, i, j)], a01 = p[nidx(P, i, j + 1)];
    const double a10 = p[nidx(P, i + 1, j)], a11 = p[nidx(P, i + 1, j + 1)];
    double Dpx = 0.0, Dpy = 0.0;
    Dpx = Dpx + -1.0 * a00; Dpy = Dpy + -1.0 * a00;
    Dpx = Dpx + -1.0 * a01; Dpy = Dpy + 1.0 * a01;
    Dpx = Dpx + 1.0 * a10;  Dpy = Dpy + -1.0 * a10;
    Dpx = Dpx + 1.0 * a11;  Dpy = Dpy + 1.0 * a11;
    Dpx = Dpx * (0.5 / P.dx);
    Dpy = Dpy * (0.5 / P.dy);
    const double Gammainv = P.gamm / (P.gamm - 1.0);
    const double thinv = rho[e] / rhoY[e];
    const double Y = rhoY[e] / rho[e];
    const double coeff = Gammainv * rhoY[e] * Y;
    const double U0 = -P.dt * coeff * Dpx, V0 = -P.dt * coeff * Dpy, W0 = -P.dt * coeff * 0.0;
    const double ds = dSdy(P, S0n, j);
    const CorCoef c = cor_coef(P, Y, ds);
    const double U = c.denom * (c.uu * U0 + c.uv * V0 + c.uw * W0);
    const double V = c.denom * (c.vu * U0 + c.vv * V0 + c.vw * W0);
    rhou[e] = rhou[e] + thinv * U;
    const double rv = rhov[e] + thinv * V;
    rhov[e] = rv;
    rhow[e] = rhow[e] + 0.0;
    rhoX[e] = rhoX[e] + (-updt_chi * P.dt * ds * rv);
}

// p2_full = 0; p2_full[2:-2,2:-2] = x.reshape(iny, inx).T  (second_projection.py:241-245)
__global__ void k_scatter(ProjDev P, const double *x, double *pfull) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.ncx * P.ncy) return;
    const int i = (int)(e / P.ncy), j = (int)(e - (long long)i * P.ncy);
    const int inx = P.ncx - 4, iny = P.ncy - 4;
    double v = 0.0;
    if (i >= 2 && i < 2 + inx && j >= 2 && j < 2 + iny) v = x[(long long)(j - 2) * inx + (i - 2)];
    pfull[e] = v;
}

__global__ void k_add(long long n, double *a, const double *b) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e < n) a[e] += b[e];
}

// ---- explicit parts (second_projection.py:22-92) --------------------------------
struct ExplDev {
    double u0, v0, w0;       // background wind
    double c1, cv, c2;       // coriolis strengths (ud.coriolis_strength)
    double ak;               // 1 - is_ArakawaKonor
};

// divergence_nodes without the 1/dt (:39) and scale_wall_node_values(rhs, 2.0) (:40,
// second_projection.py:433-474, wall_scale)
__global__ void k_fw_div(ProjDev P, const double *rho, const double *rhou, const double *rhov, const double *rhoY,
                         double *div) {
    const int nix = P.icx - 1, niy = P.icy - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy) return;
    const int a = (int)(e / niy), b = (int)(e - (long long)a * niy);
    auto qu = [&](int i, int j) { return rhou[cidx(P, i, j)] * (rhoY[cidx(P, i, j)] / rho[cidx(P, i, j)]); };
    auto qv = [&](int i, int j) { return rhov[cidx(P, i, j)] * (rhoY[cidx(P, i, j)] / rho[cidx(P, i, j)]); };
    const double d0 = (qu(a + 1, b) - qu(a, b)) / P.dx;
    const double d1 = (qu(a + 1, b + 1) - qu(a, b + 1)) / P.dx;
    const double e0 = (qv(a, b + 1) - qv(a, b)) / P.dy;
    const double e1 = (qv(a + 1, b + 1) - qv(a + 1, b)) / P.dy;
    double v = 0.5 * (d0 + d1) + 0.5 * (e0 + e1);
    {
        const int c[2] = {a, b}, n[2] = {nix, niy}, wall[2] = {P.xbc, P.ybc};
        v *= wall_scale(2, c, n, wall, 2.0);
    }
    div[e] = v;
}

// momenta and rhoX of euler_forward_non_advective (:45-64), every cell, old p2
__global__ void k_fw_cells(ProjDev P, ExplDev X, const double *p2, double *rho, double *rhou, double *rhov,
                           double *rhow, const double *rhoY, double *rhoX, const double *S0c, const double *S0n) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy) return;
    const int i = (int)(e / P.icy), j = (int)(e - (long long)i * P.icy);
    const double a00 = p2[nidx(P, i, j)], a01 = p2[nidx(P, i, j + 1)];
    const double a10 = p2[nidx(P, i + 1, j)], a11 = p2[nidx(P, i + 1, j + 1)];
    double Dpx = 0.0, Dpy = 0.0;
    Dpx = Dpx + -1.0 * a00; Dpy = Dpy + -1.0 * a00;
    Dpx = Dpx + -1.0 * a01; Dpy = Dpy + 1.0 * a01;
    Dpx = Dpx + 1.0 * a10;  Dpy = Dpy + -1.0 * a10;
    Dpx = Dpx + 1.0 * a11;  Dpy = Dpy + 1.0 * a11;
    Dpx = Dpx * (0.5 / P.dx);
    Dpy = Dpy * (0.5 / P.dy);
    const double Gammainv = P.gamm / (P.gamm - 1.0);
    const double r = rho[e], rY = rhoY[e], ru = rhou[e], rv = rhov[e], rw = rhow[e];
    const double rhoYovG = Gammainv * rY;
    const double dbuoy = rY * (rhoX[e] / r);
    const double drhou = ru - X.u0 * r, drhov = rv - X.v0 * r, drhow = rw - X.w0 * r;
    const double v = rv / r;
    const double ch1 = X.c1, cv = X.cv, ch2 = X.c2;
    rhou[e] = ru - P.dt * (rhoYovG * Dpx - ch2 * drhov + cv * drhow);
    rhov[e] = rv - P.dt * (rhoYovG * Dpy + (P.g / P.Msq) * dbuoy * P.nonhydro - ch1 * drhow + ch2 * drhou) * X.ak;
    rhoX[e] = (r * (r / rY - S0c[e])) - P.dt * (v * dSdy(P, S0n, j)) * r;
}

// p2[1:-1,1:-1] += compressibility * (-dt * dpidP * div) (:45-47, :66-69)
__global__ void k_fw_nodes(ProjDev P, const double *rhoY, const double *div, double *p2) {
    const int nix = P.icx - 1, niy = P.icy - 1;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)nix * niy) return;
    const int a = (int)(e / niy), b = (int)(e - (long long)a * niy);
    const double ex = P.gamm - 2.0;
    const double box = pow(rhoY[cidx(P, a, b)], ex) + pow(rhoY[cidx(P, a + 1, b)], ex) +
                       pow(rhoY[cidx(P, a, b + 1)], ex) + pow(rhoY[cidx(P, a + 1, b + 1)], ex);
    const double dpidP = ((P.gamm - 1.0) / P.Msq) * box / 4.0;
    const double dp = 0.0 - P.dt * dpidP * div[e];
    double &q = p2[nidx(P, a + 1, b + 1)];
    q = q + P.compressibility * dp;
}

// euler_backward_non_advective_expl_part (:82-90), every cell
__global__ void k_ex_cells(ProjDev P, ExplDev X, double *rho, double *rhou, double *rhov, double *rhow,
                           const double *rhoY, const double *rhoX, const double *S0n) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)P.icx * P.icy) return;
    const int j = (int)(e % P.icy);
    const double r = rho[e];
    const double dbuoy = rhoY[e] * (rhoX[e] / r);
    double U = rhou[e], V = (P.nonhydro * rhov[e]) - P.dt * (P.g / P.Msq) * dbuoy, W = rhow[e];
    U = U + (-1.0 * X.u0) * r;
    V = V + (-1.0 * X.v0) * r;
    W = W + (-1.0 * X.w0) * r;
    const CorCoef c = cor_coef(P, rhoY[e] / r, dSdy(P, S0n, j));
    const double U2 = c.denom * (c.uu * U + c.uv * V + c.uw * W);
    const double V2 = c.denom * (c.vu * U + c.vv * V + c.vw * W);
    const double W2 = c.denom * (c.wu * U + c.wv * V + c.ww * W);
    rhou[e] = U2 + (1.0 * X.u0) * r;
    rhov[e] = V2 + (1.0 * X.v0) * r;
    rhow[e] = W2 + (1.0 * X.w0) * r;
}

}  // namespace bella

using namespace bella;

static int grid1(long long n) { return (int)((n + 255) / 256); }

// One projection between its preparation and its correction: the geometry and
// the scratch it keeps in the workspace (ws->proj_buf), and the operator it set.
struct Proj2DState {
    ProjDev P;
    long long ncell, nnode, nisc, nin;
    double *wplus0, *dinv_isc, *rhs_isc, *hx, *hy, *cxx, *cyy, *cxy, *cyx, *hc, *dinv, *bvec, *xvec, *pfull;
    bella_op2d op;
};

static int proj2d_check(const bella_ws *ws, const bella_proj2d *a) {
    if (!ws || !a) return BELLA_EINVAL;
    if (a->inx < 3 || a->iny < 3 || !a->rho || !a->rhou || !a->rhov || !a->rhow || !a->rhoY || !a->rhoX ||
        !a->p2 || !a->hydro_rhoY0 || !a->S0n || !a->strat_inv)
        return BELLA_EINVAL;
    if (a->precond != 0 && (a->precond != 1 || !a->y_wall)) return BELLA_EINVAL;
    return BELLA_OK;
}

// Steps 1-5 of the projection up to the solve: boundary data of the coefficient
// state, ghost nodes and correction with the old p2, coefficients and diagonal,
// divergence right-hand side, the operator set in ws (second_projection.py:113-205).
static int proj2d_prepare(bella_ws *ws, const bella_proj2d *a, Proj2DState &S, cudaStream_t s) {
    ProjDev &P = S.P;
    P.icx = a->inx + 3; P.icy = a->iny + 3;
    P.ncx = a->inx + 4; P.ncy = a->iny + 4;
    P.xbc = a->x_wall ? 1 : 0; P.ybc = a->y_wall ? 1 : 0;
    P.dx = a->dx; P.dy = a->dy; P.dt = a->dt; P.Msq = a->Msq; P.g = a->g; P.gamm = a->gamm;
    P.nonhydro = a->nonhydro; P.compressibility = a->compressibility;
    P.wh1 = a->dt * a->coriolis[0]; P.wv = a->dt * a->coriolis[1]; P.wh2 = a->dt * a->coriolis[2];
    P.is_compressible = a->is_compressible;
    const long long ncell = (long long)P.icx * P.icy, nnode = (long long)P.ncx * P.ncy;
    const long long nisc = (long long)(P.icx - 1) * (P.icy - 1);
    const long long nin = (long long)a->inx * a->iny, npk = (long long)(a->inx + 1) * (a->iny + 1);
    S.ncell = ncell; S.nnode = nnode; S.nisc = nisc; S.nin = nin;
    // scratch: wplus0, dinv_isc, rhs_isc, packed hx, hy, cxx, cyy, cxy, cyx, hc, dinv, b, x, pfull
    const size_t need = (size_t)(ncell + 2 * nisc + 6 * npk + 4 * nin + nnode);
    if (ws->proj_cap < need) {
        cudaFree(ws->proj_buf);
        ws->proj_buf = nullptr;
        ws->proj_cap = 0;
        if (cudaMalloc(&ws->proj_buf, need * sizeof(double)) != cudaSuccess) return BELLA_ECUDA;
        ws->proj_cap = need;
    }
    double *q = ws->proj_buf;
    S.wplus0 = q; q += ncell;
    S.dinv_isc = q; q += nisc;
    S.rhs_isc = q; q += nisc;
    S.hx = q; q += npk;
    S.hy = q; q += npk;
    S.cxx = q; q += npk;
    S.cyy = q; q += npk;
    S.cxy = q; q += npk;
    S.cyx = q; q += npk;
    S.hc = q; q += nin;
    S.dinv = q; q += nin;
    S.bvec = q; q += nin;
    S.xvec = q; q += nin;
    S.pfull = q;

    const bool has0 = a->rho0 != nullptr;
    // 1. coefficient state: set_explicit_boundary_data(Sol0 or Sol)   (:113-118)
    double *C[6] = {has0 ? a->rho0 : a->rho, has0 ? a->rhou0 : a->rhou, has0 ? a->rhov0 : a->rhov,
                    has0 ? a->rhow0 : a->rhow, has0 ? a->rhoY0 : a->rhoY, has0 ? a->rhoX0 : a->rhoX};
    k_bd_x<<<grid1(P.icy), 256, 0, s>>>(P, C[0], C[1], C[2], C[3], C[4], C[5]);
    k_bd_y<<<grid1(P.icx), 256, 0, s>>>(P, C[0], C[1], C[2], C[3], C[4], C[5], a->hydro_rhoY0, a->strat_inv);
    // 2. ghost nodes of p2 and correction with the old p2 (:130-132)
    k_ghost_x<<<grid1(P.ncy), 256, 0, s>>>(P, a->p2);
    k_ghost_y<<<grid1(P.ncx), 256, 0, s>>>(P, a->p2);
    k_correction<<<grid1(ncell), 256, 0, s>>>(P, a->p2, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX,
                                             a->S0n, 0.0);
    k_bd_x<<<grid1(P.icy), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX);
    k_bd_y<<<grid1(P.icx), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0,
                                       a->strat_inv);
    // 3. coefficients (wplus from the coefficient state, Coriolis factors from Sol) and diagonal
    k_coeff_cells<<<grid1(ncell), 256, 0, s>>>(P, C[0], C[4], a->rho, a->rhoY, a->S0n, S.wplus0, S.hx, S.hy, S.cxx,
                                              S.cyy, S.cxy, S.cyx);
    k_coeff_nodes<<<grid1(nisc), 256, 0, s>>>(P, C[4], S.wplus0, S.dinv_isc, S.hc, S.dinv);
    // 4. divergence right-hand side (:134-170, :214)
    k_zero_ghost_momenta<<<grid1(P.icx), 256, 0, s>>>(P, a->rhou, a->rhov, a->rhow);
    k_divergence<<<grid1(nisc), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhoY, S.dinv_isc, S.rhs_isc, S.bvec);
    ws->launches += 11;
    if (a->rhs_out) cudaMemcpyAsync(a->rhs_out, S.rhs_isc, nisc * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (cudaGetLastError() != cudaSuccess) return BELLA_ECUDA;
    // 5. operator (:175, :205); cross planes only when Coriolis is on
    const bool cross = (a->coriolis[0] != 0.0 || a->coriolis[1] != 0.0 || a->coriolis[2] != 0.0);
    const bool hc_on = !(a->is_compressible == 0 && a->compressibility == 0.0);
    bella_op2d &op = S.op;
    op.nx = a->inx; op.ny = a->iny; op.x_wall = a->x_wall; op.y_wall = a->y_wall; op.dx = a->dx; op.dy = a->dy;
    op.hplusx = S.hx; op.hplusy = S.hy; op.hcenter = hc_on ? S.hc : nullptr;
    op.cxx = S.cxx; op.cyy = S.cyy; op.cxy = cross ? S.cxy : nullptr; op.cyx = cross ? S.cyx : nullptr;
    op.diag_inv = S.dinv;
    return bella_op2d_set(ws, &op, s);
}

// Step 6 after the solve: p2_full, ghost nodes, correction with updt_chi = 1,
// p2 += p2_full, ghosts, boundary data (:241-277).
static int proj2d_finish(bella_ws *ws, const bella_proj2d *a, const Proj2DState &S, cudaStream_t s) {
    const ProjDev &P = S.P;
    k_scatter<<<grid1(S.nnode), 256, 0, s>>>(P, S.xvec, S.pfull);
    k_ghost_x<<<grid1(P.ncy), 256, 0, s>>>(P, S.pfull);
    k_ghost_y<<<grid1(P.ncx), 256, 0, s>>>(P, S.pfull);
    k_correction<<<grid1(S.ncell), 256, 0, s>>>(P, S.pfull, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX,
                                               a->S0n, 1.0);
    k_add<<<grid1(S.nnode), 256, 0, s>>>(S.nnode, a->p2, S.pfull);
    k_ghost_x<<<grid1(P.ncy), 256, 0, s>>>(P, a->p2);
    k_ghost_y<<<grid1(P.ncx), 256, 0, s>>>(P, a->p2);
    k_bd_x<<<grid1(P.icy), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX);
    k_bd_y<<<grid1(P.icx), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0,
                                       a->strat_inv);
    ws->launches += 9;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" int bella_projection2d(bella_ws *ws, const bella_proj2d *a, const bella_solve_opts *opts,
                                  bella_solve_stats *stats, void *stream) {
    int rc = proj2d_check(ws, a);
    if (rc != BELLA_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    Proj2DState S;
    rc = proj2d_prepare(ws, a, S, s);
    if (rc != BELLA_OK) return rc;
    bella_solve_opts o;
    if (opts) o = *opts; else bella_solve_opts_default(&o);
    o.x0_zero = 1;
    int st;
    if (a->precond == 1) {
        // the workspace's background solve, re-derived from this call's coefficients
        // (made anew when the grid or a boundary kind changed)
        if (!ws->sp_cache || bella_spectral2d_update(ws->sp_cache, &S.op, stream) != BELLA_OK) {
            bella_spectral3d_destroy(ws->sp_cache);
            ws->sp_cache = nullptr;
            rc = bella_spectral2d_create(&ws->sp_cache, &S.op, ws->device, stream);
            if (rc != BELLA_OK) return rc;
        }
        st = bella_fbicgstab_pc(ws, ws->sp_cache, nullptr, 0, S.bvec, S.xvec, &o, stats, stream);
    } else {
        st = bella_bicgstab(ws, S.bvec, S.xvec, &o, stats, stream);
    }
    if (st < 0) return st;
    rc = proj2d_finish(ws, a, S, s);
    return rc != BELLA_OK ? rc : st;
}

extern "C" int bella_projection2d_batched(bella_ws *const *ws, const bella_proj2d *const *args, int nmembers,
                                          const bella_solve_opts *opts, int config, bella_solve_stats *stats,
                                          void *stream) {
    if (!ws || !args || nmembers < 1) return BELLA_EINVAL;
    for (int m = 0; m < nmembers; ++m) {
        const int rc = proj2d_check(ws[m], args[m]);
        if (rc != BELLA_OK) return rc;
        if (args[m]->precond != 0) return BELLA_EINVAL;      // the batched solve is plain BiCGStab
        for (int k = 0; k < m; ++k)
            if (ws[k] == ws[m]) return BELLA_EINVAL;          // every member keeps its own workspace
    }
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<Proj2DState> S(nmembers);
    std::vector<const double *> b(nmembers);
    std::vector<double *> x(nmembers);
    for (int m = 0; m < nmembers; ++m) {
        const int rc = proj2d_prepare(ws[m], args[m], S[m], s);
        if (rc != BELLA_OK) return rc;
        b[m] = S[m].bvec;
        x[m] = S[m].xvec;
    }
    const int st = bella_bicgstab_batched(ws, nmembers, b.data(), x.data(), opts, config, stats, stream);
    if (st < 0) return st;
    for (int m = 0; m < nmembers; ++m) {
        const int rc = proj2d_finish(ws[m], args[m], S[m], s);
        if (rc != BELLA_OK) return rc;
    }
    return st;
}

static int expl_setup(const bella_expl2d *a, ProjDev &P, ExplDev &X) {
    if (!a || a->inx < 3 || a->iny < 3 || !a->rho || !a->rhou || !a->rhov || !a->rhow || !a->rhoY || !a->rhoX ||
        !a->S0n || !a->hydro_rhoY0 || !a->strat_inv || !(a->dt > 0.0))
        return BELLA_EINVAL;
    P.icx = a->inx + 3; P.icy = a->iny + 3;
    P.ncx = a->inx + 4; P.ncy = a->iny + 4;
    P.xbc = a->x_wall ? 1 : 0; P.ybc = a->y_wall ? 1 : 0;
    P.dx = a->dx; P.dy = a->dy; P.dt = a->dt; P.Msq = a->Msq; P.g = a->g; P.gamm = a->gamm;
    P.nonhydro = a->nonhydro; P.compressibility = a->compressibility;
    P.wh1 = a->dt * a->coriolis[0]; P.wv = a->dt * a->coriolis[1]; P.wh2 = a->dt * a->coriolis[2];
    P.is_compressible = a->is_compressible;
    X.u0 = a->wind[0]; X.v0 = a->wind[1]; X.w0 = a->wind[2];
    X.c1 = a->coriolis[0]; X.cv = a->coriolis[1]; X.c2 = a->coriolis[2];
    X.ak = 1.0 - (double)a->is_ArakawaKonor;
    return BELLA_OK;
}

extern "C" int bella_euler_forward2d(const bella_expl2d *a, void *stream) {
    ProjDev P;
    ExplDev X;
    int rc = expl_setup(a, P, X);
    if (rc != BELLA_OK) return rc;
    if (!a->p2 || !a->rhs_out || !a->S0c) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    const long long ncell = (long long)P.icx * P.icy, nisc = (long long)(P.icx - 1) * (P.icy - 1);
    // divergence of the momenta with the wall ghosts zeroed (:39-42), into mpv.rhs
    k_zero_ghost_momenta<<<grid1(P.icx), 256, 0, s>>>(P, a->rhou, a->rhov, a->rhow);
    k_fw_div<<<grid1(nisc), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhoY, a->rhs_out);
    // momenta and rhoX with the old p2 (:45-64), then p2 (:66-69)
    k_fw_cells<<<grid1(ncell), 256, 0, s>>>(P, X, a->p2, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX,
                                           a->S0c, a->S0n);
    k_fw_nodes<<<grid1(nisc), 256, 0, s>>>(P, a->rhoY, a->rhs_out, a->p2);
    // ghost nodes and boundary data (:71-72)
    k_ghost_x<<<grid1(P.ncy), 256, 0, s>>>(P, a->p2);
    k_ghost_y<<<grid1(P.ncx), 256, 0, s>>>(P, a->p2);
    k_bd_x<<<grid1(P.icy), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX);
    k_bd_y<<<grid1(P.icx), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0,
                                       a->strat_inv);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

extern "C" int bella_expl_part2d(const bella_expl2d *a, void *stream) {
    ProjDev P;
    ExplDev X;
    int rc = expl_setup(a, P, X);
    if (rc != BELLA_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const long long ncell = (long long)P.icx * P.icy;
    k_ex_cells<<<grid1(ncell), 256, 0, s>>>(P, X, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->S0n);
    k_bd_x<<<grid1(P.icy), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX);
    k_bd_y<<<grid1(P.icx), 256, 0, s>>>(P, a->rho, a->rhou, a->rhov, a->rhow, a->rhoY, a->rhoX, a->hydro_rhoY0,
                                       a->strat_inv);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}
