// bella_advect.cuh -- arithmetic of the reference's advection (explicit.py,
// recovery.py, numerical_flux.py) in 2D and 3D, one face, cell or boundary line
// at a time.
//
// Every function is __host__ __device__: the kernels of bella_advect.cu call them
// one thread per item, and the host build of the same header (tests/advect_host.cpp)
// checks them against the oracle on the CPU.  Arithmetic follows the reference
// operation by operation (FP64), so that the sweeps reproduce it to rounding.
//
// Layout: cell arrays C order over (x, y) or (x, y, z), ic[] cells per axis with
// two ghost layers.  A sweep along axis s works on lines along s; the line index
// runs over the other axes in the order the reference's flips leave them (the
// cyclic successors of s: sweep x over (y, z), y over (z, x), z over (x, y)), so
// the face arrays of sweep s are the reference's elem.sfx / sfy / sfz: (lines,
// n_s + 1), face f between cells f-1 and f of a line.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define BELLA_HD __host__ __device__ __forceinline__
#else
#define BELLA_HD inline
#endif

namespace bella {

struct AdvGeom {
    int nd;                    // 2 or 3
    int ic[3];                 // cells incl. ghosts per axis (ic[2] = 1 in 2D)
    int bc[3];                 // 0 periodic, 1 wall
    double d[3];               // dx, dy, dz
    double g, gamm;            // gravity along y (ud.gravity_strength[1]), th.gamm
    int is_compressible;
};

struct AdvFields {             // rho, rhou, rhov, rhow, rhoY, rhoX
    double *f[6];
};

struct AdvFaces {              // face arrays of one sweep: rho, rhou, rhov, rhow, rhoY (mass flux), rhoX
    double *f[6];
};

BELLA_HD int adv_ns(const AdvGeom &G, int s) { return G.ic[s]; }
// the other axes of sweep s, outer first
BELLA_HD int adv_a1(const AdvGeom &G, int s) { return (s + 1) % G.nd; }
BELLA_HD int adv_a2(const AdvGeom &G, int s) { return (s + 2) % G.nd; }
BELLA_HD int adv_nl(const AdvGeom &G, int s) {
    return G.nd == 2 ? G.ic[adv_a1(G, s)] : G.ic[adv_a1(G, s)] * G.ic[adv_a2(G, s)];
}
BELLA_HD void adv_coords(const AdvGeom &G, int s, int l, int c, int *x) {
    x[2] = 0;
    x[s] = c;
    if (G.nd == 2) {
        x[adv_a1(G, s)] = l;
    } else {
        const int n2 = G.ic[adv_a2(G, s)];
        x[adv_a1(G, s)] = l / n2;
        x[adv_a2(G, s)] = l - (l / n2) * n2;
    }
}
BELLA_HD long long adv_flat(const AdvGeom &G, const int *x) {
    return G.nd == 2 ? (long long)x[0] * G.ic[1] + x[1] : ((long long)x[0] * G.ic[1] + x[1]) * G.ic[2] + x[2];
}
// cell (line l, position c) of sweep s -> flat index of the state arrays
BELLA_HD long long adv_cell(const AdvGeom &G, int s, int l, int c) {
    int x[3];
    adv_coords(G, s, l, c, x);
    return adv_flat(G, x);
}
BELLA_HD long long adv_face(const AdvGeom &G, int s, int l, int f) {
    return (long long)l * (adv_ns(G, s) + 1) + f;
}
// every coordinate of the line off the outer ghost layer (the reference's inner_idx)
BELLA_HD bool adv_inner_line(const AdvGeom &G, int s, int l) {
    int x[3];
    adv_coords(G, s, l, 1, x);
    for (int a = 0; a < G.nd; ++a)
        if (a != s && (x[a] < 1 || x[a] > G.ic[a] - 2)) return false;
    return true;
}

// set_explicit_boundary_data along axis s for line l of the other axis
// (boundary.py:7-216): wrap or symmetric (rhov negative-symmetric, rhow left as it
// is) when there is no gravity along s, else the hydrostatic reflection along y
// (boundary.py:56-132 with get_gravity_padding :248-281, non-Lamb branch)
BELLA_HD void adv_bd_line(const AdvGeom &G, int s, int l, const AdvFields &F, const double *hydro_rhoY0,
                          const double *strat_inv) {
    const int n = adv_ns(G, s);
    if (s != 1 || G.g == 0.0) {
        for (int q = 0; q < 6; ++q) {
            double *a = F.f[q];
            if (G.bc[s] == 0) {
                a[adv_cell(G, s, l, 0)] = a[adv_cell(G, s, l, n - 4)];
                a[adv_cell(G, s, l, 1)] = a[adv_cell(G, s, l, n - 3)];
                a[adv_cell(G, s, l, n - 2)] = a[adv_cell(G, s, l, 2)];
                a[adv_cell(G, s, l, n - 1)] = a[adv_cell(G, s, l, 3)];
            } else {
                if (q == 3) continue;
                const double sg = (q == 2) ? -1.0 : 1.0;
                a[adv_cell(G, s, l, 1)] = sg * a[adv_cell(G, s, l, 2)];
                a[adv_cell(G, s, l, 0)] = sg * a[adv_cell(G, s, l, 3)];
                a[adv_cell(G, s, l, n - 2)] = sg * a[adv_cell(G, s, l, n - 3)];
                a[adv_cell(G, s, l, n - 1)] = sg * a[adv_cell(G, s, l, n - 4)];
            }
        }
        return;
    }
    double *rho = F.f[0], *rhou = F.f[1], *rhov = F.f[2], *rhow = F.f[3], *rhoY = F.f[4], *rhoX = F.f[5];
    const double gamm = G.gamm, gm1 = gamm - 1.0, gm1inv = 1.0 / gm1, Gamma = gm1 / gamm;
    const int igy = 2;
    double direction = -1.0;
    int offset = 0;
    for (int side = 0; side < 2; ++side) {
        direction *= -1.0;
        for (int cur = igy - 1; cur >= 0; --cur) {
            const int cur_idx = cur + offset * ((n - 1) - 2 * cur);
            const long long L = adv_cell(G, s, l, (int)(cur_idx + direction));
            const long long S_ = adv_cell(G, s, l, (int)(offset * n + direction * (2 * igy - (1 - offset) - cur)));
            const long long I = adv_cell(G, s, l, cur_idx);
            const double Y_last = rhoY[L] / rho[L];
            const double rhoYv_image = -rhov[S_] * rhoY[S_] / rho[S_];
            const double S = strat_inv[cur_idx];
            const double dpi = direction * (Gamma * G.g) * 0.5 * G.d[1] * (1.0 / Y_last + S);
            const double rY = (G.is_compressible == 1) ? pow(pow(rhoY[L], gm1) + dpi, gm1inv) : hydro_rhoY0[cur_idx];
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

// primitive q / rho where rho != 0, else 0 (Vars.primitives, variable.py:56-86)
BELLA_HD double adv_prim(double q, double rho) { return rho != 0.0 ? q / rho : 0.0; }

// primitives u, v, w, Y, X of one cell, the advecting velocity U (recovery.py:60-62:
// face mass fluxes averaged over the cell's two faces, divided by rhoY; zero off the
// inner cells) and the differences to the right neighbour (recovery.py:70-76; zero
// at the last cell), for the quantities u, v, w, X and 1/Y
struct AdvCell {
    double p[5];     // u, v, w, X, Y
    double d[5];     // right difference of u, v, w, X, 1/Y
    double U;
};

BELLA_HD void adv_prims(const AdvGeom &G, int s, int l, int c, const AdvFields &F, double *p) {
    const long long e = adv_cell(G, s, l, c);
    const double rho = F.f[0][e];
    p[0] = adv_prim(F.f[1][e], rho);
    p[1] = adv_prim(F.f[2][e], rho);
    p[2] = adv_prim(F.f[3][e], rho);
    p[3] = adv_prim(F.f[5][e], rho);
    p[4] = adv_prim(F.f[4][e], rho);
}

BELLA_HD void adv_cell_state(const AdvGeom &G, int s, int l, int c, const AdvFields &F, const double *mflux,
                             AdvCell &A) {
    const int ns = adv_ns(G, s);
    adv_prims(G, s, l, c, F, A.p);
    A.U = 0.0;
    if (c >= 1 && c <= ns - 2 && adv_inner_line(G, s, l))
        A.U = 0.5 * (mflux[adv_face(G, s, l, c)] + mflux[adv_face(G, s, l, c + 1)]) / F.f[4][adv_cell(G, s, l, c)];
    if (c < ns - 1) {
        double r[5];
        adv_prims(G, s, l, c + 1, F, r);
        for (int k = 0; k < 4; ++k) A.d[k] = r[k] - A.p[k];
        A.d[4] = 1.0 / r[4] - 1.0 / A.p[4];
    } else {
        for (int k = 0; k < 5; ++k) A.d[k] = 0.0;
    }
}

// limited slope of cell c from its own and its left neighbour's right differences
// (recovery.py:144-238, limiter NONE: the mean; zero at the first and last cell)
BELLA_HD void adv_slopes(int ns, int c, const AdvCell &left, const AdvCell &self, double *S) {
    for (int k = 0; k < 5; ++k) S[k] = (c >= 1 && c <= ns - 2) ? 0.5 * (left.d[k] + self.d[k]) : 0.0;
}

// an interface state of a cell (recovery.py:80-113) turned conservative with the
// face mass density rhoY_face (get_conservatives, recovery.py:241-262), then back
// to the primitives the flux uses (hll_solver's primitives, numerical_flux.py:80-81).
// side +1: the cell's right face (Lefts), -1: its left face (Rights)
BELLA_HD void adv_face_state(const AdvCell &A, const double *S, double lmbda, double side, double rhoY_face,
                             double *out /* u, v, w, X, Y */) {
    double q[5];
    for (int k = 0; k < 4; ++k) {
        const double amp = side > 0.0 ? 0.5 * S[k] * (1.0 - lmbda * A.U) : -0.5 * S[k] * (1.0 + lmbda * A.U);
        q[k] = A.p[k] + 1 * amp;
    }
    const double ampY = side > 0.0 ? 0.5 * S[4] * (1.0 - lmbda * A.U) : -0.5 * S[4] * (1.0 + lmbda * A.U);
    const double Yf = 1.0 / (1.0 / A.p[4] + 1 * ampY);
    const double rho = rhoY_face / Yf;
    const double ru = q[0] * rho, rv = q[1] * rho, rw = q[2] * rho, rY = Yf * rho, rX = q[3] * rho;
    out[0] = adv_prim(ru, rho);
    out[1] = adv_prim(rv, rho);
    out[2] = adv_prim(rw, rho);
    out[3] = adv_prim(rX, rho);
    out[4] = adv_prim(rY, rho);
}

// fluxes of face f (1 <= f <= n_s - 1) of line l (recovery.do + hll_solver,
// numerical_flux.py:48-99): upwind by the sign of the face mass flux
BELLA_HD void adv_face_flux(const AdvGeom &G, int s, int l, int f, const AdvFields &F, double lmbda,
                            const AdvFaces &out) {
    const int ns = adv_ns(G, s);
    const double *mflux = out.f[4];
    AdvCell a0, a1, a2;                       // cells f-2 (if any), f-1, f
    adv_cell_state(G, s, l, f - 1, F, mflux, a1);
    adv_cell_state(G, s, l, f, F, mflux, a2);
    if (f >= 2) adv_cell_state(G, s, l, f - 2, F, mflux, a0);
    else for (int k = 0; k < 5; ++k) a0.d[k] = 0.0;
    double SL[5], SR[5];
    adv_slopes(ns, f - 1, a0, a1, SL);
    adv_slopes(ns, f, a1, a2, SR);
    // face mass density between cells f-1 and f (recovery.py:117-119), vel = u, v or w of the sweep
    const long long eL = adv_cell(G, s, l, f - 1), eR = adv_cell(G, s, l, f);
    const double rYL = F.f[4][eL], rYR = F.f[4][eR];
    const double vL = a1.p[s], vR = a2.p[s];
    const double face = 0.5 * (rYL + rYR) - 1 * 0.5 * lmbda * (vR * rYR - vL * rYL);
    double PL[5], PR[5];
    adv_face_state(a1, SL, lmbda, 1.0, face, PL);
    adv_face_state(a2, SR, lmbda, -1.0, face, PR);
    const double fm = mflux[adv_face(G, s, l, f)];
    const double sg = fm > 0.0 ? 1.0 : (fm < 0.0 ? -1.0 : 0.0);
    const double upl = 0.5 * (1.0 + sg), upr = (1.0 - upl);
    const long long o = adv_face(G, s, l, f);
    out.f[1][o] = fm * (upl / PL[4] * PL[0] + upr / PR[4] * PR[0]);
    out.f[0][o] = fm * (upl / PL[4] * 1.0 + upr / PR[4] * 1.0);
    out.f[2][o] = fm * (upl / PL[4] * PL[1] + upr / PR[4] * PR[1]);
    out.f[3][o] = fm * (upl / PL[4] * PL[2] + upr / PR[4] * PR[2]);
    out.f[5][o] = fm * (upl / PL[4] * PL[3] + upr / PR[4] * PR[3]);
}

// conservative update of cell c of line l (explicit.py:146-151)
BELLA_HD void adv_update_cell(const AdvGeom &G, int s, int l, int c, const AdvFields &F, const AdvFaces &fl,
                              double lmbda) {
    const long long e = adv_cell(G, s, l, c), a = adv_face(G, s, l, c), b = adv_face(G, s, l, c + 1);
    for (int q = 0; q < 6; ++q) F.f[q][e] = F.f[q][e] + lmbda * (fl.f[q][a] - fl.f[q][b]);
}

// face mass flux of inner face f of line l of sweep s (recompute_advective_fluxes,
// numerical_flux.py:5-46): rhoY times the sweep's velocity on the two cells of the
// face, weighted across it by (0.5, 1, 0.5) over -1..+1 in 2D (sum of weights 4)
// and by [[1,2,1],[2,4,2],[1,2,1]] over the two other axes in 3D (sum 32).
// Inner faces: f in 1..n_s-1 on lines off the outer ghost layer.
BELLA_HD double adv_mass(const AdvGeom &G, int s, int l, int f, const AdvFields &F) {
    int x0[3];
    adv_coords(G, s, l, f - 1, x0);
    const int a1 = adv_a1(G, s), a2 = adv_a2(G, s);
    const double *mom = F.f[1 + s];
    const double w1[3] = {0.5, 1.0, 0.5};
    const double K2[3][3] = {{1, 2, 1}, {2, 4, 2}, {1, 2, 1}};
    double sum = 0.0;
    for (int p = 0; p < 2; ++p)
        for (int q = 0; q < 3; ++q)
            for (int r = 0; r < (G.nd == 3 ? 3 : 1); ++r) {
                int x[3] = {x0[0], x0[1], x0[2]};
                x[s] += p;
                x[a1] += q - 1;
                double w = w1[q];
                if (G.nd == 3) {
                    x[a2] += r - 1;
                    w = K2[q][r];
                }
                const long long e = adv_flat(G, x);
                sum += w * (F.f[4][e] * mom[e] / F.f[0][e]);
            }
    return sum / (G.nd == 3 ? 32.0 : 4.0);
}

}  // namespace bella

namespace bella {

// The sweep sequences of advect (explicit.py:5-74) and advect_rk (:160-257),
// written once over an executor that runs one pass over all lines / faces / cells
// (kernel launches on the device, loops on the host):
//   ex.bd(s)              boundary data along axis s
//   ex.faces(s, lmbda)    fluxes of every inner face of sweep s
//   ex.update(s, lmbda)   conservative update of every cell by sweep s
//   ex.pwchi(lmbda)       rhoX update of the y sweep (advect_rk's Sol.pwchi)
template <class Ex>
void adv_sweep(Ex &ex, int s, double lmbda) {          // explicit_step_and_flux (explicit.py:77-158)
    ex.bd(s);
    ex.faces(s, lmbda);
    ex.update(s, lmbda);
    ex.bd(s);
}

template <class Ex>
void adv_strang(Ex &ex, const AdvGeom &G, double dt, int odd) {
    const double h = 0.5 * dt;
    const int nd = G.nd;
    if (odd) {
        for (int s = 0; s < nd; ++s) adv_sweep(ex, s, h / G.d[s]);
        for (int s = nd - 1; s >= 0; --s) adv_sweep(ex, s, h / G.d[s]);
    } else {
        for (int s = nd - 1; s >= 0; --s) adv_sweep(ex, s, h / G.d[s]);
        for (int s = 0; s < nd; ++s) adv_sweep(ex, s, h / G.d[s]);
    }
    for (int s = 0; s < nd; ++s) ex.bd(s);
}

template <class Ex>
void adv_rk(Ex &ex, const AdvGeom &G, double dt) {
    for (int s = 0; s < G.nd; ++s) {                    // fluxes from the start state (lmbda 0 in recovery)
        ex.bd(s);
        ex.faces(s, 0.0);
        ex.bd(s);
    }
    for (int s = 0; s < G.nd; ++s) ex.update(s, dt / G.d[s]);
    ex.pwchi(dt / G.d[1]);
    for (int s = 0; s < G.nd; ++s) ex.bd(s);
}

}  // namespace bella
