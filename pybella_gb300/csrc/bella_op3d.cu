// bella_op3d.cu -- 3D 27-point nodal Helmholtz operator and its fused
// BiCGStab kernels (sm_103a).
//
// The operator is the arithmetic of the reference's lap3D
// (laplacian.py:898-1026) in cell-flux form.  Every cell computes its
// four-edge difference sums
//   Gx = (c100+c110+c101+c111) - (c000+c010+c001+c011)   (and Gy, Gz alike)
// over its eight corner nodes cXYZ, and its fluxes
//   Fx = Ax Gx + Cxz Gz,  Fy = Ay Gy,  Fz = Az Gz - Czx Gx
// with Ax = hplusx/(16 dx^2), ..., Cxz = corrf hplusx/(16 dx dz),
// Czx = corrf hplusz/(16 dx dz) (the Coriolis cross terms of
// laplacian.py:987-997,1020-1021).  A node sums, per axis, the fluxes of the
// four cells on its + side minus the four on its - side, adds hcenter*u and
// scales by diag_inv (laplacian.py:1017-1024).  Unknowns are all inner nodes
// in C order over (x, y, z); a periodic axis wraps with the duplicated seam
// (wrap distance n-1) and a wall zeroes the outer cell planes, the
// conventions of the reference's 2D operator (the 3D glue of the reference,
// second_projection.py:183-203, cannot run).
//
// A CTA of 256 threads (32 along z, 8 along y) owns a 4x8x32 node tile:
// it stages the stencil input u with a one-node halo (6x10x34) in dynamic
// shared memory (u is formed on the fly from the Krylov vectors), computes the
// 5x9x33 cell fluxes into shared memory and writes 4 nodes per thread.
#include "bella_internal.cuh"

namespace bella {

constexpr int T3X = 4, T3Y = 8, T3Z = 32;
constexpr int H3X = T3X + 2, H3Y = T3Y + 2, H3Z = T3Z + 2;
constexpr int C3X = T3X + 1, C3Y = T3Y + 1, C3Z = T3Z + 1;
constexpr int NU3 = H3X * H3Y * H3Z;      // 2040 halo values
constexpr int NC3 = C3X * C3Y * C3Z;      // 1485 cells

template <typename T>
struct Op3D {
    int nx, ny, nz;
    const T *ax, *ay, *az, *cxz, *czx;     // cell planes (nx+1)(ny+1)(nz+1)
    const T *dinv, *hc;                    // node planes
};

template <typename T>
struct StArgs3 {
    const T *x, *b;
    T *y;
    const T *r, *rh;
    T *p0, *p1, *v0, *v1;
};

template <typename T>
size_t smem3d_bytes() { return sizeof(T) * (NU3 + 3 * NC3); }

// ---- operator packing -------------------------------------------------------
__global__ void k_pack3d_cells(bella_op3d op, double *a64, float *a32, dfloat *adf) {
    const long long nxc = op.nx + 1, nyc = op.ny + 1, nzc = op.nz + 1;
    const long long ncell = nxc * nyc * nzc;
    const double c = 1.0 / 16.0;
    const double wx = c / (op.dx * op.dx), wy = c / (op.dy * op.dy), wz = c / (op.dz * op.dz);
    const double wxz = op.corrf * c / (op.dx * op.dz);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ncell;
         e += (long long)gridDim.x * blockDim.x) {
        const long long ck = e % nzc, t = e / nzc, cj = t % nyc, ci = t / nyc;
        double hx = op.hplusx[e], hy = op.hplusy[e], hz = op.hplusz[e];
        // walls: the outer cell planes never couple (laplacian.py:933-965)
        const bool wall = (op.x_wall && (ci == 0 || ci == nxc - 1)) || (op.y_wall && (cj == 0 || cj == nyc - 1)) ||
                          (op.z_wall && (ck == 0 || ck == nzc - 1));
        if (wall) { hx = 0.0; hy = 0.0; hz = 0.0; }
        const double v[5] = {wx * hx, wy * hy, wz * hz, wxz * hx, wxz * hz};
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            a64[q * ncell + e] = v[q];
            a32[q * ncell + e] = (float)v[q];
            adf[q * ncell + e] = dfloat(v[q]);
        }
    }
}

// node planes and the left null weights z = w/diag_inv (trapezoid weight 1/2
// per periodic axis on the duplicated seam)
__global__ void k_pack3d_nodes(bella_op3d op, double *dinv64, float *dinv32, dfloat *dinvdf, double *hc64,
                               float *hc32, dfloat *hcdf, double *z64) {
    const long long n = (long long)op.nx * op.ny * op.nz;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const long long k = g % op.nz, t = g / op.nz, j = t % op.ny, i = t / op.ny;
        const double d = op.diag_inv[g];
        const double h = op.hcenter ? op.hcenter[g] : 0.0;
        dinv64[g] = d; dinv32[g] = (float)d; dinvdf[g] = dfloat(d);
        hc64[g] = h; hc32[g] = (float)h; hcdf[g] = dfloat(h);
        double w = 1.0;
        if (!op.x_wall && (i == 0 || i == op.nx - 1)) w *= 0.5;
        if (!op.y_wall && (j == 0 || j == op.ny - 1)) w *= 0.5;
        if (!op.z_wall && (k == 0 || k == op.nz - 1)) w *= 0.5;
        z64[g] = w / d;
    }
}

__device__ __forceinline__ int wrap3(int g, int n) {
    if (g < 0) return g + n - 1;
    if (g == n) return 1;
    return g;
}

// ---- fused stencil ---------------------------------------------------------------
template <typename T, int MODE, bool CROSS, bool HC>
__global__ void __launch_bounds__(256)
k_stencil3d(Op3D<T> op, StArgs3<T> a, KState *ks, double *partials, unsigned *counter) {
    using AccT = typename Acc<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *su = reinterpret_cast<T *>(smem_raw);          // [H3X][H3Y][H3Z]
    T *sfx = su + NU3;                                // [C3X][C3Y][C3Z]
    T *sfy = sfx + NC3;
    T *sfz = sfy + NC3;

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
    const int nx = op.nx, ny = op.ny, nz = op.nz;
    const int tx = (nx + T3X - 1) / T3X, ty = (ny + T3Y - 1) / T3Y, tz = (nz + T3Z - 1) / T3Z;
    const long long ntiles = (long long)tx * ty * tz;
    const int tid = threadIdx.x;
    const T *pin = par ? a.p1 : a.p0;
    T *pout = par ? a.p0 : a.p1;
    const T *vold = par ? a.v1 : a.v0;
    T *vnew = par ? a.v0 : a.v1;
    const T *vin = (MODE == M_PDIR) ? vold : vnew;
    T *yout = (MODE == M_PDIR) ? vnew : a.y;
    const long long nyz = (long long)ny * nz;
    const long long cyz = (long long)(ny + 1) * (nz + 1);

    AccT acc0, acc1, acc2;
    acc0.zero(); acc1.zero(); acc2.zero();

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tzi = (int)(tile % tz);
        const long long rest = tile / tz;
        const int tyi = (int)(rest % ty), txi = (int)(rest / ty);
        const int i0 = txi * T3X, j0 = tyi * T3Y, k0 = tzi * T3Z;
        // 1. u on the tile + halo
        for (int e = tid; e < NU3; e += 256) {
            const int la = e / (H3Y * H3Z), rem = e - la * (H3Y * H3Z), lb = rem / H3Z, ld = rem - lb * H3Z;
            const int gi = wrap3(i0 - 1 + la, nx), gj = wrap3(j0 - 1 + lb, ny), gk = wrap3(k0 - 1 + ld, nz);
            T u = 0;
            if (gi < nx && gj < ny && gk < nz) {
                const long long g = gi * nyz + (long long)gj * nz + gk;
                if (MODE == M_APPLY || MODE == M_RESID) {
                    u = a.x[g];
                } else if (MODE == M_PDIR) {
                    const T rg = a.r[g];
                    u = first ? rg : rg + beta * (pin[g] - omega * vin[g]);
                    const bool owner = la >= 1 && la <= T3X && lb >= 1 && lb <= T3Y && ld >= 1 && ld <= T3Z &&
                                       i0 - 1 + la < nx && j0 - 1 + lb < ny && k0 - 1 + ld < nz;
                    if (owner) pout[g] = u;
                } else {
                    u = a.r[g] - alpha * vin[g];
                }
            }
            su[e] = u;
        }
        __syncthreads();
        // 2. cell fluxes
        for (int e = tid; e < NC3; e += 256) {
            const int la = e / (C3Y * C3Z), rem = e - la * (C3Y * C3Z), lb = rem / C3Z, ld = rem - lb * C3Z;
            const int ci = i0 + la, cj = j0 + lb, ck = k0 + ld;
            T fx = 0, fy = 0, fz = 0;
            if (ci <= nx && cj <= ny && ck <= nz) {
                const long long c = ci * cyz + (long long)cj * (nz + 1) + ck;
                const int b0 = (la * H3Y + lb) * H3Z + ld;
                const T c000 = su[b0], c001 = su[b0 + 1];
                const T c010 = su[b0 + H3Z], c011 = su[b0 + H3Z + 1];
                const T c100 = su[b0 + H3Y * H3Z], c101 = su[b0 + H3Y * H3Z + 1];
                const T c110 = su[b0 + H3Y * H3Z + H3Z], c111 = su[b0 + H3Y * H3Z + H3Z + 1];
                const T gx = ((c100 + c110) + (c101 + c111)) - ((c000 + c010) + (c001 + c011));
                const T gy = ((c010 + c110) + (c011 + c111)) - ((c000 + c100) + (c001 + c101));
                const T gz = ((c001 + c101) + (c011 + c111)) - ((c000 + c100) + (c010 + c110));
                fx = op.ax[c] * gx;
                fy = op.ay[c] * gy;
                fz = op.az[c] * gz;
                if (CROSS) {
                    fx += op.cxz[c] * gz;
                    fz = fz - op.czx[c] * gx;
                }
            }
            sfx[e] = fx;
            sfy[e] = fy;
            sfz[e] = fz;
        }
        __syncthreads();
        // 3. nodes: thread (ld, lb) computes x-planes la = 0..T3X-1
        const int ld = tid & 31, lb = tid >> 5;
#pragma unroll
        for (int la = 0; la < T3X; ++la) {
            const int gi = i0 + la, gj = j0 + lb, gk = k0 + ld;
            if (gi < nx && gj < ny && gk < nz) {
                const long long g = gi * nyz + (long long)gj * nz + gk;
                const int c0 = (la * C3Y + lb) * C3Z + ld;                 // cell (la, lb, ld)
                const int dx_ = C3Y * C3Z, dy_ = C3Z;
                const T xs = ((sfx[c0 + dx_] + sfx[c0 + dx_ + dy_]) + (sfx[c0 + dx_ + 1] + sfx[c0 + dx_ + dy_ + 1])) -
                             ((sfx[c0] + sfx[c0 + dy_]) + (sfx[c0 + 1] + sfx[c0 + dy_ + 1]));
                const T ys = ((sfy[c0 + dy_] + sfy[c0 + dx_ + dy_]) + (sfy[c0 + dy_ + 1] + sfy[c0 + dx_ + dy_ + 1])) -
                             ((sfy[c0] + sfy[c0 + dx_]) + (sfy[c0 + 1] + sfy[c0 + dx_ + 1]));
                const T zs = ((sfz[c0 + 1] + sfz[c0 + dx_ + 1]) + (sfz[c0 + dy_ + 1] + sfz[c0 + dx_ + dy_ + 1])) -
                             ((sfz[c0] + sfz[c0 + dx_]) + (sfz[c0 + dy_] + sfz[c0 + dx_ + dy_]));
                const T u = su[((la + 1) * H3Y + lb + 1) * H3Z + ld + 1];
                T s = (xs + ys) + zs;
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
    if (MODE == M_RESID) ks->dot_aux2 = tot[0];
    else if (MODE == M_PDIR) finalize_pdir(ks, tot[0]);
    else finalize_sdir(ks, tot[0], tot[1], tot[2]);
}

// ---- host side ----------------------------------------------------------------------
template <typename T> static Op3D<T> make_op3(bella_ws *ws, const T *planes, const T *dinv, const T *hc) {
    const size_t nc = (size_t)(ws->nx + 1) * (ws->ny + 1) * (ws->nz + 1);
    Op3D<T> o;
    o.nx = ws->nx; o.ny = ws->ny; o.nz = ws->nz;
    o.ax = planes; o.ay = planes + nc; o.az = planes + 2 * nc; o.cxz = planes + 3 * nc; o.czx = planes + 4 * nc;
    o.dinv = dinv; o.hc = hc;
    return o;
}
static Op3D<double> op3_of(bella_ws *ws, double *) { return make_op3<double>(ws, ws->a64, ws->dinv64, ws->hc64); }
static Op3D<float> op3_of(bella_ws *ws, float *) { return make_op3<float>(ws, ws->a32, ws->dinv32, ws->hc32); }
static Op3D<dfloat> op3_of(bella_ws *ws, dfloat *) { return make_op3<dfloat>(ws, ws->adf, ws->dinvdf, ws->hcdf); }

int stencil3d_grid(int nx, int ny, int nz) {
    const long long tiles = (long long)((nx + T3X - 1) / T3X) * ((ny + T3Y - 1) / T3Y) * ((nz + T3Z - 1) / T3Z);
    const long long cap = (long long)num_sms() * 4;
    return (int)(tiles < cap ? tiles : cap);
}

template <typename T, int MODE, bool CROSS, bool HC>
static void launch3_one(bella_ws *ws, const StArgs3<T> &a, cudaStream_t s) {
    static bool attr_set[64] = {false};
    const size_t sm = smem3d_bytes<T>();
    const int dev = ws->device & 63;
    if (!attr_set[dev]) {   // > 48 KB of dynamic shared memory needs the opt-in (set per device)
        cudaFuncSetAttribute(k_stencil3d<T, MODE, CROSS, HC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr_set[dev] = true;
    }
    k_stencil3d<T, MODE, CROSS, HC><<<ws->grid_stencil, 256, sm, s>>>(op3_of(ws, (T *)nullptr), a, ws->ks,
                                                                        ws->partials, ws->counter);
}

template <typename T, int MODE>
static void launch3(bella_ws *ws, const StArgs3<T> &a, cudaStream_t s) {
    const int pk = MODE == M_PDIR ? PK_PDIR : MODE == M_SDIR ? PK_SDIR : MODE == M_RESID ? PK_RESID : -1;
    if (pk >= 0) prof_begin(ws, pk, s);
    if (ws->cross) {
        if (ws->has_hc) launch3_one<T, MODE, true, true>(ws, a, s);
        else            launch3_one<T, MODE, true, false>(ws, a, s);
    } else {
        if (ws->has_hc) launch3_one<T, MODE, false, true>(ws, a, s);
        else            launch3_one<T, MODE, false, false>(ws, a, s);
    }
    if (pk >= 0) prof_end(ws, pk, s);
    ws->launches++;
}

int op3d_pack(bella_ws *ws, const bella_op3d *op, cudaStream_t s) {
    const long long ncell = (long long)(op->nx + 1) * (op->ny + 1) * (op->nz + 1);
    int g = (int)((ncell + 255) / 256);
    if (g > num_sms() * 8) g = num_sms() * 8;
    k_pack3d_cells<<<g, 256, 0, s>>>(*op, ws->a64, ws->a32, ws->adf);
    k_pack3d_nodes<<<g, 256, 0, s>>>(*op, ws->dinv64, ws->dinv32, ws->dinvdf, ws->hc64, ws->hc32, ws->hcdf,
                                     ws->z64);
    ws->launches += 2;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

void op3d_apply(bella_ws *ws, int prec, const void *x, void *y, cudaStream_t s) {
    if (prec == 0) {
        StArgs3<double> a = {};
        a.x = (const double *)x; a.y = (double *)y;
        launch3<double, M_APPLY>(ws, a, s);
    } else {
        StArgs3<float> a = {};
        a.x = (const float *)x; a.y = (float *)y;
        launch3<float, M_APPLY>(ws, a, s);
    }
}

void op3d_resid(bella_ws *ws, int prec, const void *x, const void *b, void *r, cudaStream_t s) {
    if (prec == 0) {
        StArgs3<double> a = {};
        a.x = (const double *)x; a.b = (const double *)b; a.y = (double *)r;
        launch3<double, M_RESID>(ws, a, s);
    } else {
        StArgs3<float> a = {};
        a.x = (const float *)x; a.b = (const float *)b; a.y = (float *)r;
        launch3<float, M_RESID>(ws, a, s);
    }
}

void op3d_iteration(bella_ws *ws, int prec, cudaStream_t s) {
    if (prec == 2) {
        StArgs3<dfloat> a = {};
        a.r = ws->rdf; a.rh = ws->rhdf; a.y = ws->tdf;
        a.p0 = ws->pdf[0]; a.p1 = ws->pdf[1]; a.v0 = ws->vdf[0]; a.v1 = ws->vdf[1];
        launch3<dfloat, M_PDIR>(ws, a, s);
        launch3<dfloat, M_SDIR>(ws, a, s);
        launch_update<dfloat>(ws, s);
    } else if (prec == 0) {
        StArgs3<double> a = {};
        a.r = ws->r64k; a.rh = ws->rh64; a.y = ws->t64;
        a.p0 = ws->p64[0]; a.p1 = ws->p64[1]; a.v0 = ws->v64[0]; a.v1 = ws->v64[1];
        launch3<double, M_PDIR>(ws, a, s);
        launch3<double, M_SDIR>(ws, a, s);
        launch_update<double>(ws, s);
    } else {
        StArgs3<float> a = {};
        a.r = ws->r32; a.rh = ws->rh32; a.y = ws->t32;
        a.p0 = ws->p32[0]; a.p1 = ws->p32[1]; a.v0 = ws->v32[0]; a.v1 = ws->v32[1];
        launch3<float, M_PDIR>(ws, a, s);
        launch3<float, M_SDIR>(ws, a, s);
        launch_update<float>(ws, s);
    }
}

}  // namespace bella
