// bella_op2d.cu -- 2D 9-point nodal Helmholtz operator and the fused
// BiCGStab kernels built on it (sm_103a).
//
// The operator is the reference's lap2D_gather_new (laplacian.py:546-746)
// rewritten in cell-flux form: every cell c computes, from the diagonal
// differences d1 = BR - TL and d2 = TR - BL,
//   Gx = (d1 + d2)/2 = ((TR-TL)+(BR-BL))/2,  Gy = (d1 - d2)/2 = ((BL-TL)+(BR-TR))/2
//   Fx = Axx*Gx + Axy*Gy,  Fy = Ayy*Gy + Ayx*Gx,  P = Fx + Fy,  M = Fx - Fy
// once, and each node sums its four cells
//   y = dinv * ( (M[TR] - M[BL]) + (P[BR] - P[TL]) + hc*u )
//     = dinv * ( Fx[TR]+Fx[BR]-Fx[TL]-Fx[BL] + Fy[BL]+Fy[BR]-Fy[TL]-Fy[TR] + hc*u )
// which is algebraically the reference's Dxx+Dyy+Dyx+Dxy+hcenter*p scaled by
// diag_inv (laplacian.py:721-739); 9 additions per node instead of 13.  Walls are folded into the cell planes
// (zeroed outer cell column/row, laplacian.py:691-713); the periodic wrap
// with the duplicated seam (laplacian.py:595-638) is done on the halo load.
// The LAMB_BDRY variant (lap2D_numba_test with its padding and the kernel_9pt
// stencil, laplacian.py:531-543, 749-868) is the same operator on the same cell
// planes with a mirrored y boundary on the halo load and no cell zeroed.
//
// A CTA owns a 64x16 node tile: it stages the tile plus a one-node halo of
// the stencil input u in shared memory (computing u on the fly from the
// Krylov vectors where the mode asks for it), computes the 65x17 cell
// fluxes into shared memory, then writes the 64x16 outputs and accumulates
// the inner products of the iteration in double-float registers.  The grid
// is a multiple of the SM count and loops over tiles.
#include "bella_internal.cuh"

namespace bella {

template <typename T>
struct StArgs {
    const T *x;      // APPLY / RESID input
    const T *b;      // RESID right-hand side
    T *y;            // APPLY / RESID / SDIR output
    const T *r, *rh;
    T *p0, *p1, *v0, *v1;
};

// --------------------------------------------------------------------------
// operator packing: reference operands -> cell planes (FP64 and FP32)
// --------------------------------------------------------------------------
__global__ void k_pack2d_cells(bella_op2d op, double *a64, float *a32, dfloat *adf, int cross) {
    const int nx = op.nx, ny = op.ny;
    const size_t ncell = (size_t)(nx + 1) * (ny + 1);
    const double oodx = 1.0 / op.dx, oody = 1.0 / op.dy;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell;
         c += (size_t)gridDim.x * blockDim.x) {
        const int cj = (int)(c / (nx + 1)), ci = (int)(c - (size_t)cj * (nx + 1));
        double hx = op.hplusx[c], hy = op.hplusy[c];
        // wall handling: the outer cell column/row never couples (laplacian.py:691-713)
        if (op.x_wall && (ci == 0 || ci == nx)) { hx = 0.0; hy = 0.0; }
        if (op.y_wall == 1 && (cj == 0 || cj == ny)) { hx = 0.0; hy = 0.0; }   // not for the mirror (2)
        const double axx = 0.5 * oodx * oodx * op.cxx[c] * hx;
        const double ayy = 0.5 * oody * oody * op.cyy[c] * hy;
        const double axy = cross ? 0.5 * oodx * oody * (op.cxy ? op.cxy[c] : 0.0) * hy : 0.0;
        const double ayx = cross ? 0.5 * oodx * oody * (op.cyx ? op.cyx[c] : 0.0) * hx : 0.0;
        a64[c] = axx; a64[ncell + c] = ayy; a64[2 * ncell + c] = axy; a64[3 * ncell + c] = ayx;
        a32[c] = (float)axx; a32[ncell + c] = (float)ayy;
        a32[2 * ncell + c] = (float)axy; a32[3 * ncell + c] = (float)ayx;
        if (adf) {   // double-float planes (absent in the allocation-free path)
            adf[c] = dfloat(axx); adf[ncell + c] = dfloat(ayy);
            adf[2 * ncell + c] = dfloat(axy); adf[3 * ncell + c] = dfloat(ayx);
        }
    }
}

// node planes; z = left null weights / diag_inv (trapezoid weight 1/2 on the
// duplicated periodic seam), used to project the pseudo-incompressible
// solution onto the operator's range.
__global__ void k_pack2d_nodes(bella_op2d op, double *dinv64, float *dinv32, double *hc64,
                               float *hc32, double *z64, dfloat *dinvdf, dfloat *hcdf) {
    const int nx = op.nx, ny = op.ny;
    const size_t n = (size_t)nx * ny;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
         g += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(g / nx), i = (int)(g - (size_t)j * nx);
        const double d = op.diag_inv[g];
        const double h = op.hcenter ? op.hcenter[g] : 0.0;
        dinv64[g] = d; dinv32[g] = (float)d;
        hc64[g] = h;   hc32[g] = (float)h;
        if (dinvdf) { dinvdf[g] = dfloat(d); hcdf[g] = dfloat(h); }
        double w = 1.0;
        if (!op.x_wall && (i == 0 || i == nx - 1)) w *= 0.5;
        if (op.y_wall == 0 && (j == 0 || j == ny - 1)) w *= 0.5;
        z64[g] = w / d;
    }
}

// --------------------------------------------------------------------------
// fused stencil kernel
// --------------------------------------------------------------------------
template <typename T, int MODE, bool CROSS, bool HC>
__global__ void __launch_bounds__(NTHREADS, MINB)
k_stencil2d(Op2D<T> op, StArgs<T> a, KState *ks, double *partials, unsigned *counter) {
    using AccT = typename Acc<T>::type;
    __shared__ T su[TY + 2][TX + 2];
    __shared__ T sfx[TY + 1][TX + 1];
    __shared__ T sfy[TY + 1][TX + 1];

    int par = 0;
    bool first = false;
    T alpha = 0, beta = 0, omega = 0;
    if (MODE == M_PDIR || MODE == M_SDIR) {
        if (ks->done) return;
        par = ks->iter & 1;
        first = (ks->iter == 0);
        alpha = (T)ks->alpha;
        beta = (T)ks->beta;
        omega = (T)ks->omega;
    }
    const int nx = op.nx, ny = op.ny;
    const int tilesx = (nx + TX - 1) / TX, tilesy = (ny + TY - 1) / TY;
    const int ntiles = tilesx * tilesy;
    const int tid = threadIdx.x + threadIdx.y * BX;
    const T *pin = par ? a.p1 : a.p0;
    T *pout = par ? a.p0 : a.p1;
    const T *vold = par ? a.v1 : a.v0;
    T *vnew = par ? a.v0 : a.v1;
    const T *vin = (MODE == M_PDIR) ? vold : vnew;   // SDIR reads the fresh v
    T *yout = (MODE == M_PDIR) ? vnew : a.y;

    AccT acc0, acc1, acc2;
    acc0.zero(); acc1.zero(); acc2.zero();

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tyi = tile / tilesx, txi = tile - tyi * tilesx;
        const int j0 = tyi * TY, i0 = txi * TX;
        // 1. stencil input u on the tile + one-node halo (wrap: duplicated seam)
#pragma unroll
        for (int e = tid; e < (TY + 2) * (TX + 2); e += NTHREADS) {
            const int la = e / (TX + 2), lb = e - la * (TX + 2);
            int gj = j0 - 1 + la, gi = i0 - 1 + lb;
            if (gj < 0) gj = op.ymirror ? 1 : gj + ny - 1;          // mirror (LAMB_BDRY) or wrap
            else if (gj == ny) gj = op.ymirror ? ny - 2 : 1;
            if (gi < 0) gi += nx - 1; else if (gi == nx) gi = 1;
            T u = 0;
            if (gj < ny && gi < nx) {
                const size_t g = (size_t)gj * nx + gi;
                if (MODE == M_APPLY || MODE == M_RESID) {
                    u = a.x[g];
                } else if (MODE == M_PDIR) {
                    const T rg = a.r[g];
                    u = first ? rg : rg + beta * (pin[g] - omega * vin[g]);
                    const bool owner = (la >= 1 && la <= TY && lb >= 1 && lb <= TX &&
                                        j0 - 1 + la < ny && i0 - 1 + lb < nx);
                    if (owner) pout[g] = u;
                } else {  // M_SDIR: s = r - alpha v
                    u = a.r[g] - alpha * vin[g];
                }
            }
            su[la][lb] = u;
        }
        __syncthreads();
        // 2. cell fluxes
#pragma unroll
        for (int e = tid; e < (TY + 1) * (TX + 1); e += NTHREADS) {
            const int la = e / (TX + 1), lb = e - la * (TX + 1);
            const int cj = j0 + la, ci = i0 + lb;
            T fx = 0, fy = 0;
            if (cj <= ny && ci <= nx) {
                const size_t c = (size_t)cj * (nx + 1) + ci;
                const T tl = su[la][lb], tr = su[la][lb + 1];
                const T bl = su[la + 1][lb], br = su[la + 1][lb + 1];
                const T d1 = br - tl, d2 = tr - bl;
                const T gx = half_of(d1 + d2);
                const T gy = half_of(d1 - d2);
                fx = op.axx[c] * gx;
                fy = op.ayy[c] * gy;
                if (CROSS) {
                    fx += op.axy[c] * gy;
                    fy += op.ayx[c] * gx;
                }
            }
            sfx[la][lb] = fx + fy;   // P
            sfy[la][lb] = fx - fy;   // M
        }
        __syncthreads();
        // 3. node outputs
        const int lb = threadIdx.x;
#pragma unroll
        for (int k = 0; k < TY / BY; ++k) {
            const int la = threadIdx.y + k * BY;
            const int gj = j0 + la, gi = i0 + lb;
            if (gj < ny && gi < nx) {
                const size_t g = (size_t)gj * nx + gi;
                const T u = su[la + 1][lb + 1];
                // cells around node (la+1, lb+1) of the halo tile: TL (la, lb), TR (la, lb+1),
                // BL (la+1, lb), BR (la+1, lb+1); sfx holds P, sfy holds M
                T s = (sfy[la][lb + 1] - sfy[la + 1][lb]) + (sfx[la + 1][lb + 1] - sfx[la][lb]);
                if (HC) s += op.hc[g] * u;
                T yv = s * op.dinv[g];
                if (MODE == M_RESID) {
                    yv = a.b[g] - yv;
                    acc0.add_prod(yv, yv);
                } else if (MODE == M_PDIR) {
                    acc0.add_prod(a.rh[g], yv);
                } else if (MODE == M_SDIR) {
                    acc0.add_prod(yv, u);
                    acc1.add_prod(yv, yv);
                    acc2.add_prod(u, u);
                }
                yout[g] = yv;
            }
        }
        __syncthreads();
    }
    if (MODE == M_APPLY) return;

    double v[3] = {acc0.value(), acc1.value(), acc2.value()};
    double tot[3];
    if (!grid_sum<3>(v, partials, counter, tot)) return;
    if (tid != 0) return;
    if (MODE == M_RESID) {
        ks->dot_aux2 = tot[0];
    } else if (MODE == M_PDIR) {
        finalize_pdir(ks, tot[0]);
    } else {
        finalize_sdir(ks, tot[0], tot[1], tot[2]);
    }
}

// --------------------------------------------------------------------------
// host launchers
// --------------------------------------------------------------------------
template <typename T>
static Op2D<T> make_op(bella_ws *ws);

template <>
Op2D<double> make_op<double>(bella_ws *ws) {
    const size_t nc = (size_t)(ws->nx + 1) * (ws->ny + 1);
    Op2D<double> o;
    o.nx = ws->nx; o.ny = ws->ny; o.ymirror = ws->ymirror;
    o.axx = ws->a64; o.ayy = ws->a64 + nc; o.axy = ws->a64 + 2 * nc; o.ayx = ws->a64 + 3 * nc;
    o.dinv = ws->dinv64; o.hc = ws->hc64;
    return o;
}

template <>
Op2D<dfloat> make_op<dfloat>(bella_ws *ws) {
    const size_t nc = (size_t)(ws->nx + 1) * (ws->ny + 1);
    Op2D<dfloat> o;
    o.nx = ws->nx; o.ny = ws->ny; o.ymirror = ws->ymirror;
    o.axx = ws->adf; o.ayy = ws->adf + nc; o.axy = ws->adf + 2 * nc; o.ayx = ws->adf + 3 * nc;
    o.dinv = ws->dinvdf; o.hc = ws->hcdf;
    return o;
}

template <>
Op2D<float> make_op<float>(bella_ws *ws) {
    const size_t nc = (size_t)(ws->nx + 1) * (ws->ny + 1);
    Op2D<float> o;
    o.nx = ws->nx; o.ny = ws->ny; o.ymirror = ws->ymirror;
    o.axx = ws->a32; o.ayy = ws->a32 + nc; o.axy = ws->a32 + 2 * nc; o.ayx = ws->a32 + 3 * nc;
    o.dinv = ws->dinv32; o.hc = ws->hc32;
    return o;
}

int stencil_grid(int nx, int ny) {
    const int tiles = ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
    const int cap = num_sms() * (GRID_PER_SM < 8 ? GRID_PER_SM : 8);   // partials hold MAXGRID CTAs
    return tiles < cap ? tiles : cap;
}

template <typename T, int MODE>
static void launch_mode(bella_ws *ws, const StArgs<T> &a, cudaStream_t s) {
    Op2D<T> op = make_op<T>(ws);
    dim3 blk(BX, BY);
    const int grid = ws->grid_stencil;
    const int pk = MODE == M_PDIR ? PK_PDIR : MODE == M_SDIR ? PK_SDIR : MODE == M_RESID ? PK_RESID : -1;
    if (pk >= 0) prof_begin(ws, pk, s);
    if (ws->cross) {
        if (ws->has_hc) k_stencil2d<T, MODE, true, true><<<grid, blk, 0, s>>>(op, a, ws->ks, ws->partials, ws->counter);
        else            k_stencil2d<T, MODE, true, false><<<grid, blk, 0, s>>>(op, a, ws->ks, ws->partials, ws->counter);
    } else {
        if (ws->has_hc) k_stencil2d<T, MODE, false, true><<<grid, blk, 0, s>>>(op, a, ws->ks, ws->partials, ws->counter);
        else            k_stencil2d<T, MODE, false, false><<<grid, blk, 0, s>>>(op, a, ws->ks, ws->partials, ws->counter);
    }
    if (pk >= 0) prof_end(ws, pk, s);
    ws->launches++;
}

int op2d_pack(bella_ws *ws, const bella_op2d *op, cudaStream_t s) {
    const size_t ncell = (size_t)(op->nx + 1) * (op->ny + 1);
    int g = (int)((ncell + 255) / 256);
    if (g > num_sms() * 8) g = num_sms() * 8;
    k_pack2d_cells<<<g, 256, 0, s>>>(*op, ws->a64, ws->a32, ws->adf, ws->cross);
    k_pack2d_nodes<<<g, 256, 0, s>>>(*op, ws->dinv64, ws->dinv32, ws->hc64, ws->hc32, ws->z64, ws->dinvdf,
                                     ws->hcdf);
    ws->launches += 2;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

void op2d_apply(bella_ws *ws, int prec, const void *x, void *y, cudaStream_t s) {
    if (prec == 0) {
        StArgs<double> a = {};
        a.x = (const double *)x; a.y = (double *)y;
        launch_mode<double, M_APPLY>(ws, a, s);
    } else {
        StArgs<float> a = {};
        a.x = (const float *)x; a.y = (float *)y;
        launch_mode<float, M_APPLY>(ws, a, s);
    }
}

void op2d_resid(bella_ws *ws, int prec, const void *x, const void *b, void *r, cudaStream_t s) {
    if (prec == 0) {
        StArgs<double> a = {};
        a.x = (const double *)x; a.b = (const double *)b; a.y = (double *)r;
        launch_mode<double, M_RESID>(ws, a, s);
    } else {
        StArgs<float> a = {};
        a.x = (const float *)x; a.b = (const float *)b; a.y = (float *)r;
        launch_mode<float, M_RESID>(ws, a, s);
    }
}

// one BiCGStab iteration: PDIR stencil, SDIR stencil, vector update
// prec: 0 FP64, 1 FP32, 2 double-float
void op2d_iteration(bella_ws *ws, int prec, cudaStream_t s) {
    if (prec == 2) {
        StArgs<dfloat> a = {};
        a.r = ws->rdf; a.rh = ws->rhdf; a.y = ws->tdf;
        a.p0 = ws->pdf[0]; a.p1 = ws->pdf[1]; a.v0 = ws->vdf[0]; a.v1 = ws->vdf[1];
        launch_mode<dfloat, M_PDIR>(ws, a, s);
        launch_mode<dfloat, M_SDIR>(ws, a, s);
        launch_update<dfloat>(ws, s);
    } else if (prec == 0) {
        StArgs<double> a = {};
        a.r = ws->r64k; a.rh = ws->rh64; a.y = ws->t64;
        a.p0 = ws->p64[0]; a.p1 = ws->p64[1]; a.v0 = ws->v64[0]; a.v1 = ws->v64[1];
        launch_mode<double, M_PDIR>(ws, a, s);
        launch_mode<double, M_SDIR>(ws, a, s);
        launch_update<double>(ws, s);
    } else {
        StArgs<float> a = {};
        a.r = ws->r32; a.rh = ws->rh32; a.y = ws->t32;
        a.p0 = ws->p32[0]; a.p1 = ws->p32[1]; a.v0 = ws->v32[0]; a.v1 = ws->v32[1];
        launch_mode<float, M_PDIR>(ws, a, s);
        launch_mode<float, M_SDIR>(ws, a, s);
        launch_update<float>(ws, s);
    }
}

}  // namespace bella
