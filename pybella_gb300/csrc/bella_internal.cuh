// bella_internal.cuh -- declarations shared by the translation units of
// libbella_gb300 (not part of the C ABI).
#pragma once
#include "bella_common.cuh"

namespace bella {

enum { M_APPLY = 0, M_RESID = 1, M_PDIR = 2, M_SDIR = 3, M_RESX = 4 };   // M_RESX: FP64 vectors, double-float arithmetic

// ---- last-block finalisers of one BiCGStab iteration -----------------------
// The control flow follows scipy's bicgstab, which the reference calls
// (second_projection.py:230): early exit when ||s|| meets the tolerance,
// convergence on ||r||, rho and omega breakdown below eps^2.  One deviation:
// the rho test is relative, |<r^,r>| < eps^2 <r^,r0>, where scipy's is
// absolute; scipy's absolute test stops solves with a small-norm right-hand
// side (||b|| ~ 4e-5 at 2049x1025) near convergence for no numerical reason.

// after v = A p:  alpha = rho / <r^, v>
// nu and the implicit Coriolis / buoyancy factors on cells (second_projection.py:609-633)
struct CorCoef { double uu, uv, uw, vu, vv, vw, wu, wv, ww, denom; };

// P: the projection parameters of either dimension (dt, g, Msq, nonhydro, wh1, wv, wh2)
template <class PD>
__device__ __forceinline__ CorCoef cor_coef(const PD &P, double Y, double strat) {
    const double nonhydro = P.nonhydro, wh1 = P.wh1, wv = P.wv, wh2 = P.wh2;
    const double nu = -P.dt * P.dt * (P.g / P.Msq) * strat * Y;
    CorCoef c;
    c.denom = 1.0 / (wh1 * wh1 + wh2 * wh2 + (nu + nonhydro) * (wv * wv + 1.0));
    c.uu = (wh1 * wh1 + nu + nonhydro);
    c.uv = nonhydro * (wh1 * wv + wh2);
    c.uw = (wh1 * wh2 - (nu + nonhydro) * wv);
    c.vu = (wh1 * wv - wh2);
    c.vv = nonhydro * (1.0 + wv * wv);
    c.vw = (wh2 * wv + wh1);
    c.wu = (wh1 * wh2 + (nu + nonhydro) * wv);
    c.wv = nonhydro * (wh2 * wv - wh1);
    c.ww = (nu + nonhydro + wh2 * wh2);
    return c;
}

// scale_wall_node_values (second_projection.py:433-474): the factor that entry c of
// a node.isc array of extents n (nd axes, two ghost layers) receives.  The reference
// walks the wall axes in order, scales row n-2 then row 1 of each, and leaves that
// axis's index at row 1, so a later wall axis scales only the entries on row 1 of
// every earlier wall axis; the other axes run over [2, n-3].
__device__ __forceinline__ double wall_scale(int nd, const int *c, const int *n, const int *wall, double f) {
    double s = 1.0;
    for (int d = 0; d < nd; ++d) {
        if (!wall[d]) continue;
        for (int t = 0; t < 2; ++t) {
            const int row = t == 0 ? n[d] - 2 : 1;
            bool hit = true;
            for (int e = 0; e < nd; ++e) {
                if (e == d) hit = hit && c[e] == row;
                else if (e < d && wall[e]) hit = hit && c[e] == 1;
                else hit = hit && c[e] >= 2 && c[e] <= n[e] - 3;
            }
            if (hit) s *= f;
        }
    }
    return s;
}

__device__ __forceinline__ void finalize_pdir(KState *ks, double rv) {
    if (!isfinite(rv)) { ks->status = BELLA_NONFINITE; ks->done = 1; return; }
    if (rv == 0.0) { ks->status = BELLA_BREAKDOWN; ks->pad[0] = 3; ks->done = 1; return; }
    ks->alpha = ks->rho / rv;
}

// after t = A s:  omega = <t,s>/<t,t>, early exit on ||s||
__device__ __forceinline__ void finalize_sdir(KState *ks, double ts, double tt, double ss) {
    ks->ss = ss;
    if (!isfinite(ss) || !isfinite(ts) || !isfinite(tt)) {
        ks->status = BELLA_NONFINITE; ks->done = 1; return;
    }
    if (sqrt(ss) <= ks->atol) { ks->early = 1; ks->omega = 0.0; return; }
    if (!(tt > 0.0)) { ks->status = BELLA_BREAKDOWN; ks->pad[0] = 4; ks->done = 1; return; }
    ks->omega = ts / tt;
}

// after x += alpha p + omega s, r = s - omega t.  rho/beta are advanced even
// when the solve stops here, so a residual replacement can continue the
// same Krylov process (k_replace_df).
__device__ __forceinline__ void finalize_update(KState *ks, double rho_new, double rr) {
    ks->iter += 1;
    if (ks->early) { ks->status = BELLA_OK; ks->done = 1; ks->rr = ks->ss; return; }
    ks->rr = rr;
    const bool finite = isfinite(rr) && isfinite(rho_new);
    if (finite && ks->omega != 0.0) {
        ks->beta = (rho_new / ks->rho) * (ks->alpha / ks->omega);
        ks->rho_prev = ks->rho;
        ks->rho = rho_new;
    }
    if (!finite) { ks->status = BELLA_NONFINITE; ks->done = 1; }
    else if (sqrt(rr) <= ks->atol) { ks->status = BELLA_OK; ks->done = 1; }
    else if (ks->iter >= ks->maxiter) { ks->status = BELLA_MAXITER; ks->done = 1; }
    else if (fabs(rho_new) < ks->rhotol * ks->rho0) { ks->status = BELLA_BREAKDOWN; ks->pad[0] = 1; ks->done = 1; }
    else if (fabs(ks->omega) < ks->rhotol) { ks->status = BELLA_BREAKDOWN; ks->pad[0] = 2; ks->done = 1; }
}

// ---- per-kernel event timing (host) -------------------------------------------
enum { PK_PDIR = 0, PK_SDIR = 1, PK_UPDATE = 2, PK_RESID = 3 };
void prof_begin(bella_ws *ws, int kind, cudaStream_t s);
void prof_end(bella_ws *ws, int kind, cudaStream_t s);
void prof_harvest(bella_ws *ws);

// ---- error reporting (host): the message bella_last_error() returns -------------
int set_err(int code, const char *what);
int cuda_check(cudaError_t e, const char *where);   // BELLA_OK or BELLA_ECUDA with the CUDA message

// ---- launchers (host) --------------------------------------------------------
int  stencil_grid(int nx, int ny);
int  vec_grid(long long n);
int  op2d_pack(bella_ws *ws, const bella_op2d *op, cudaStream_t s);
void op2d_apply(bella_ws *ws, int prec, const void *x, void *y, cudaStream_t s);
void op2d_resid(bella_ws *ws, int prec, const void *x, const void *b, void *r, cudaStream_t s);
void op2d_iteration(bella_ws *ws, int prec, cudaStream_t s);
int  stencil3d_grid(int nx, int ny, int nz);
int  op3d_pack(bella_ws *ws, const bella_op3d *op, cudaStream_t s);
void op3d_apply(bella_ws *ws, int prec, const void *x, void *y, cudaStream_t s);
void op3d_resid(bella_ws *ws, int prec, const void *x, const void *b, void *r, cudaStream_t s);
// r = b - A x and ||r||^2 of FP64 vectors, formed in double-float arithmetic (~1e-14 of |A||x|)
void op3d_resid_df(bella_ws *ws, const double *x, const double *b, double *r, cudaStream_t s);
void op3d_iteration(bella_ws *ws, int prec, cudaStream_t s);

// dimension dispatch of the prepared operator
inline void op_apply(bella_ws *ws, int prec, const void *x, void *y, cudaStream_t s) {
    if (ws->ndim == 3) op3d_apply(ws, prec, x, y, s); else op2d_apply(ws, prec, x, y, s);
}
inline void op_resid(bella_ws *ws, int prec, const void *x, const void *b, void *r, cudaStream_t s) {
    if (ws->ndim == 3) op3d_resid(ws, prec, x, b, r, s); else op2d_resid(ws, prec, x, b, r, s);
}
inline void op_iteration(bella_ws *ws, int prec, cudaStream_t s) {
    if (ws->ndim == 3) op3d_iteration(ws, prec, s); else op2d_iteration(ws, prec, s);
}
template <typename T> void launch_update(bella_ws *ws, cudaStream_t s);

// background (spectral) solve (bella_spectral.cu): out = A_bg^+ (in / diag_inv);
// two work arrays of n floats for a composed preconditioner (not used by the
// background solve itself)
int spectral_apply_dev(bella_spectral3d *sp, const float *in, float *out, cudaStream_t s);
float *spectral_work(bella_spectral3d *sp, int which);
long long spectral_size(const bella_spectral3d *sp);

// learned preconditioner (bella_cnn.cu)
// per (optional): the periodic axes of the grid; the correction is left out within
// the network's reach of a periodic seam, where its zero padding stands in for
// the wrapped neighbours
int cnn_apply_dev(bella_cnn *net, int nx, int ny, int nz, const float *in, float *out, const double *sumsq,
                  cudaStream_t s, const int *per = nullptr);

}  // namespace bella
