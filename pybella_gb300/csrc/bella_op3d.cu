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
// The stencil streams along x.  A CTA of 256 threads owns a y-z tile of
// 8 x 32 nodes (thread (ty, tz) = (tid / 32, tid % 32) owns node
// (j0 + ty, k0 + tz)) and marches through a run of node planes [xs, xe).
// Step i of a run stores u plane i+2 with its one-node y-z halo (10 x 34;
// u is formed on the fly from the Krylov vectors), computes the 9 x 33 cell
// fluxes of cell plane i+1 and finishes node plane i-1.  The x direction is
// summed once per plane and carried in registers: a cell's gradients are
// differences and sums of its two u faces, each face's sums computed once
// (Gx = S(face x) - S(face x-1), Gy = Y(x-1) + Y(x), Gz = Z(x-1) + Z(x)), and a
// node's sums are differences and sums of its two cell planes' flux partials
// (xs = X(n+1) - X(n), ys = Y(n) + Y(n+1), zs = Z(n) + Z(n+1)).  Four u planes
// and two flux planes rotate in shared memory, so the three phases of a step
// touch disjoint buffers and one barrier per step suffices.  Every global
// load is issued two steps before its use (register sets A and B serve
// alternate steps), which keeps enough bytes in flight per SM to cover the
// DRAM latency.  The runs are even shares of the (tile, plane) sequence over
// the grid (one resident wave), so a CTA's run may span two tiles.
#include "bella_internal.cuh"

namespace bella {

constexpr int S3Y = 8, S3Z = 32;
constexpr int SUY = S3Y + 2, SUZ = S3Z + 2, SUN = SUY * SUZ;    // u plane with its halo: 10 x 34
constexpr int SCY = S3Y + 1, SCZ = S3Z + 1, SCN = SCY * SCZ;    // cell plane: 9 x 33
constexpr int SU_EXTRA = SUN - 256;                             // 84 halo nodes beyond one per thread
constexpr int SC_EXTRA = SCN - 256;                             // 41 edge cells beyond one per thread
constexpr int SU_BUF = 4, SF_BUF = 2;                           // rotating u and flux planes

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
size_t smem3d_bytes() { return sizeof(T) * (SU_BUF * SUN + SF_BUF * 3 * SCN); }

// vector loads and stores; M_RESX reads and writes FP64 values (8 bytes, the size of a
// double-float) and computes in double-float
template <typename T, int MODE> __device__ __forceinline__ T ld3(const T *p) {
    if constexpr (MODE == M_RESX) return T(*reinterpret_cast<const double *>(p));
    else return *p;
}
template <typename T, int MODE> __device__ __forceinline__ void st3(T *p, T v) {
    if constexpr (MODE == M_RESX) *reinterpret_cast<double *>(p) = v.to_double();
    else *p = v;
}

template <bool B> struct Chk { static constexpr bool value = B; };

// number of input vectors u is formed from: x (APPLY, RESID), r p v (PDIR), r v (SDIR)
template <int MODE> struct In3 { static constexpr int n = MODE == M_PDIR ? 3 : MODE == M_SDIR ? 2 : 1; };

// one thread's loads for one step: the inputs of u at its own and its extra
// halo node, the coefficients of its own and its extra cell, and its node's
// diag_inv, hcenter and rhat (PDIR) or b (RESID)
template <typename T, int MODE, bool CROSS>
struct Pref3 {
    T ui[In3<MODE>::n][2];
    T cf[CROSS ? 5 : 3][2];
    T dinv, hc, aux;
};

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
// double and double-float: at least 2 resident CTAs per SM (at most 128 registers
// a thread; measured 0.74 vs 0.86 ms per double-float iteration at 257x129x257).
// FP32: no minimum (0), where the compiler keeps the matvec at 64 registers and 4
// CTAs per SM (69 us at 257x129x257); a minimum of 1 or 2 let it take 108
// registers, 2 CTAs per SM and 89 us.
template <typename T, int MODE, bool CROSS, bool HC>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 0 : 2)
k_stencil3d(Op3D<T> op, StArgs3<T> a, KState *ks, double *partials, unsigned *counter) {
    using AccT = typename Acc<T>::type;
    constexpr int NI = In3<MODE>::n, NCF = CROSS ? 5 : 3;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *su = reinterpret_cast<T *>(smem_raw);          // [SU_BUF][SUY][SUZ]
    T *sf = su + SU_BUF * SUN;                        // [SF_BUF][Fx, Fy, Fz][SCY][SCZ]

    constexpr bool KRYLOV = MODE == M_PDIR || MODE == M_SDIR;
    if (KRYLOV && ks->done) return;
    const int par = KRYLOV ? (ks->iter & 1) : 0;
    const bool first = KRYLOV && ks->iter == 0;
    const T alpha = KRYLOV ? (T)ks->alpha : T(0), beta = KRYLOV ? (T)ks->beta : T(0),
            omega = KRYLOV ? (T)ks->omega : T(0);
    const int nx = op.nx, ny = op.ny, nz = op.nz;
    const int tyn = (ny + S3Y - 1) / S3Y, tzn = (nz + S3Z - 1) / S3Z;
    const long long work = (long long)tyn * tzn * nx;          // (y-z tile, node plane) pairs
    const int tid = threadIdx.x, ty = tid >> 5, tz = tid & 31;
    const T *pin = par ? a.p1 : a.p0;
    T *pout = par ? a.p0 : a.p1;
    const T *vold = par ? a.v1 : a.v0;
    T *vnew = par ? a.v0 : a.v1;
    const T *vin = (MODE == M_PDIR) ? vold : vnew;
    T *yout = (MODE == M_PDIR) ? vnew : a.y;
    const int nyz = ny * nz;                          // node and cell counts are below 2^31 (host check)
    const int cyz = (ny + 1) * (nz + 1);
    const T *src[3] = {MODE == M_PDIR || MODE == M_SDIR ? a.r : a.x, MODE == M_PDIR ? pin : vin, vin};
    const T *coef[5] = {op.ax, op.ay, op.az, op.cxz, op.czx};

    AccT acc0, acc1, acc2;
    acc0.zero(); acc1.zero(); acc2.zero();

    Pref3<T, MODE, CROSS> A, B;
    long long lo = work * blockIdx.x / gridDim.x;
    const long long hi = work * (blockIdx.x + 1) / gridDim.x;
    while (lo < hi) {
        const long long tile = lo / nx;
        const int xs = (int)(lo - tile * nx);
        const int xe = (int)(hi - lo < nx - xs ? xs + (hi - lo) : nx);
        lo += xe - xs;
        const int j0 = (int)(tile / tzn) * S3Y, k0 = (int)(tile % tzn) * S3Z;

        // this thread's halo nodes: its own and, for tid < 84, one of the halo ring;
        // shared-memory slot and y-z offset (-1: outside the domain, u = 0 there)
        int uslot[2] = {(ty + 1) * SUZ + tz + 1, -1}, uoff[2] = {-1, -1};
        {
            int lb[2] = {ty + 1, 0}, ld[2] = {tz + 1, 0};
            if (tid < SU_EXTRA) {
                const int e = tid;
                if (e < SUZ)                { lb[1] = 0;                     ld[1] = e; }
                else if (e < 2 * SUZ)       { lb[1] = SUY - 1;               ld[1] = e - SUZ; }
                else if (e < 2 * SUZ + S3Y) { lb[1] = e - 2 * SUZ + 1;       ld[1] = 0; }
                else                        { lb[1] = e - 2 * SUZ - S3Y + 1; ld[1] = SUZ - 1; }
                uslot[1] = lb[1] * SUZ + ld[1];
            }
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int gj = wrap3(j0 - 1 + lb[w], ny), gk = wrap3(k0 - 1 + ld[w], nz);
                if (uslot[w] >= 0 && gj < ny && gk < nz) uoff[w] = gj * nz + gk;
            }
        }
        // this thread's cells: its own and, for the last 41 threads, one of the
        // tile's far edges; flux slot, slot of the cell's (y, z) = (0, 0) corner
        // node in the u plane, y-z offset of the cell (-1: outside, flux 0)
        int cslot[2] = {ty * SCZ + tz, -1}, cu[2] = {ty * SUZ + tz, 0}, coff[2] = {-1, -1};
        {
            int cb[2] = {ty, 0}, cd[2] = {tz, 0};
            if (tid >= 256 - SC_EXTRA) {
                const int e = tid - (256 - SC_EXTRA);
                if (e < SCZ) { cb[1] = SCY - 1; cd[1] = e; }
                else         { cb[1] = e - SCZ; cd[1] = SCZ - 1; }
                cslot[1] = cb[1] * SCZ + cd[1];
                cu[1] = cb[1] * SUZ + cd[1];
            }
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int cj = j0 + cb[w], ck = k0 + cd[w];
                if (cslot[w] >= 0 && cj <= ny && ck <= nz) coff[w] = cj * (nz + 1) + ck;
            }
        }
        const bool nvalid = (j0 + ty < ny) && (k0 + tz < nz);
        const int noff = (j0 + ty) * nz + (k0 + tz);
        const int c0 = ty * SCZ + tz, uc = (ty + 1) * SUZ + tz + 1;

        // sums carried from one plane to the next: per cell, the previous u plane's
        // face sums (S: the four nodes, Y: the y+1 pair minus the y pair, Z: the
        // z+1 pair minus the z pair); per node, the previous cell plane's flux
        // partials (X: sum of the four cells' Fx, Y/Z: the upper minus the lower pair)
        T fS[2], fY[2], fZ[2], nX, nY, nZ;

        // the run's interior steps (xs+1 <= i <= xe-4) have every phase active and
        // every plane in range: they are instantiated with CK = false and no checks
        auto load_u = [&](Pref3<T, MODE, CROSS> &S, int p, auto CK) {
            if (decltype(CK)::value && p > xe) return;
            const int base = wrap3(p, nx) * nyz;
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                if (uoff[w] < 0) continue;
                S.ui[0][w] = ld3<T, MODE>(src[0] + base + uoff[w]);
                if (NI > 1 && !(MODE == M_PDIR && first)) {
#pragma unroll
                    for (int q = 1; q < NI; ++q) S.ui[q][w] = src[q][base + uoff[w]];
                }
            }
        };
        auto load_cf = [&](Pref3<T, MODE, CROSS> &S, int c, auto CK) {
            if (decltype(CK)::value && (c < xs || c > xe)) return;
            const int base = c * cyz;
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                if (coff[w] < 0) continue;
#pragma unroll
                for (int q = 0; q < NCF; ++q) S.cf[q][w] = coef[q][base + coff[w]];
            }
        };
        auto load_nd = [&](Pref3<T, MODE, CROSS> &S, int n, auto CK) {
            if ((decltype(CK)::value && (n < xs || n >= xe)) || !nvalid) return;
            const int g = n * nyz + noff;
            S.dinv = op.dinv[g];
            if (HC) S.hc = op.hc[g];
            if (MODE == M_RESID || MODE == M_RESX) S.aux = ld3<T, MODE>(a.b + g);
            if (MODE == M_PDIR) S.aux = a.rh[g];
        };
        // step i: u plane i+2 -> shared memory; face sums of u plane i+1 and the
        // fluxes of cell plane i+1; flux partials of cell plane i and node plane i-1
        auto step = [&](Pref3<T, MODE, CROSS> &S, int i, auto CK) {
            constexpr bool chk = decltype(CK)::value;
            const int p = i + 2;
            if (!chk || (p >= xs - 1 && p <= xe)) {
                T *ub = su + ((p + 4) & 3) * SUN;
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    if (uslot[w] < 0) continue;
                    T u = 0;
                    if (uoff[w] >= 0) {
                        if (MODE == M_APPLY || MODE == M_RESID || MODE == M_RESX) u = S.ui[0][w];
                        else if (MODE == M_PDIR) u = first ? S.ui[0][w] : S.ui[0][w] + beta * (S.ui[1][w] - omega * S.ui[2][w]);
                        else u = S.ui[0][w] - alpha * S.ui[NI - 1][w];
                    }
                    ub[uslot[w]] = u;
                    if (MODE == M_PDIR && w == 0 && nvalid && (!chk || (p >= xs && p < xe))) pout[p * nyz + noff] = u;
                }
            }
            load_u(S, i + 4, CK);
            const int q = i + 1;                      // u plane of the faces; cell plane q spans u planes q-1, q
            if (!chk || (q >= xs - 1 && q <= xe)) {
                const T *ub = su + ((q + 4) & 3) * SUN;
                T *fb = sf + (q & 1) * (3 * SCN);
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    if (cslot[w] < 0) continue;
                    const int b0 = cu[w];
                    const T u00 = ub[b0], u01 = ub[b0 + 1], u10 = ub[b0 + SUZ], u11 = ub[b0 + SUZ + 1];
                    const T pj = u00 + u01, pj1 = u10 + u11;
                    const T s_ = pj + pj1, y_ = pj1 - pj, z_ = (u01 + u11) - (u00 + u10);
                    if (!chk || q >= xs) {
                        T fx = 0, fy = 0, fz = 0;
                        if (coff[w] >= 0) {
                            const T gx = s_ - fS[w], gy = fY[w] + y_, gz = fZ[w] + z_;
                            fx = S.cf[0][w] * gx;
                            fy = S.cf[1][w] * gy;
                            fz = S.cf[2][w] * gz;
                            if (CROSS) {
                                fx += S.cf[3][w] * gz;
                                fz = fz - S.cf[NCF - 1][w] * gx;
                            }
                        }
                        fb[cslot[w]] = fx;
                        fb[SCN + cslot[w]] = fy;
                        fb[2 * SCN + cslot[w]] = fz;
                    }
                    fS[w] = s_; fY[w] = y_; fZ[w] = z_;
                }
            }
            load_cf(S, i + 3, CK);
            const int c = i;                          // cell plane of the partials; node plane c-1
            if ((!chk || (c >= xs && c <= xe)) && nvalid) {
                const T *fb = sf + (c & 1) * (3 * SCN);
                const T *Fx = fb, *Fy = fb + SCN, *Fz = fb + 2 * SCN;
                constexpr int dy_ = SCZ;
                const T X = (Fx[c0] + Fx[c0 + 1]) + (Fx[c0 + dy_] + Fx[c0 + dy_ + 1]);
                const T Y = (Fy[c0 + dy_] + Fy[c0 + dy_ + 1]) - (Fy[c0] + Fy[c0 + 1]);
                const T Z = (Fz[c0 + 1] + Fz[c0 + dy_ + 1]) - (Fz[c0] + Fz[c0 + dy_]);
                const int n = c - 1;
                if (!chk || n >= xs) {
                    const T u = su[((n + 4) & 3) * SUN + uc];
                    T s = ((X - nX) + (nY + Y)) + (nZ + Z);
                    if (HC) s += S.hc * u;
                    T yv = s * S.dinv;
                    if (MODE == M_RESID || MODE == M_RESX) {
                        yv = S.aux - yv;
                        acc0.add_prod(yv, yv);
                    } else if (MODE == M_PDIR) {
                        acc0.add_prod(S.aux, yv);
                    } else if (MODE == M_SDIR) {
                        acc0.add_prod(yv, u);
                        acc1.add_prod(yv, yv);
                        acc2.add_prod(u, u);
                    }
                    st3<T, MODE>(yout + n * nyz + noff, yv);
                }
                nX = X; nY = Y; nZ = Z;
            }
            load_nd(S, i + 1, CK);
            __syncthreads();
        };

        const Chk<true> checked;
        const Chk<false> steady;
        load_u(A, xs - 1, checked);
        load_u(B, xs, checked);
        int i = xs - 3;                               // steps xs-3 .. xe; A serves xs-3, xs-1, ...
        for (; i <= xe && i < xs + 1; i += 2) {
            step(A, i, checked);
            if (i + 1 <= xe) step(B, i + 1, checked);
        }
        for (; i + 1 <= xe - 4; i += 2) {
            step(A, i, steady);
            step(B, i + 1, steady);
        }
        for (; i <= xe; i += 2) {
            step(A, i, checked);
            if (i + 1 <= xe) step(B, i + 1, checked);
        }
    }
    if (MODE == M_APPLY) return;
    double v[3] = {acc0.value(), acc1.value(), acc2.value()};
    double tot[3];
    if (!grid_sum<3>(v, partials, counter, tot)) return;
    if (tid != 0) return;
    if (MODE == M_RESID || MODE == M_RESX) ks->dot_aux2 = tot[0];
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

// number of (y-z tile, node plane) pairs the stencil's runs share out
static long long stencil3d_work(int nx, int ny, int nz) {
    return (long long)((ny + S3Y - 1) / S3Y) * ((nz + S3Z - 1) / S3Z) * nx;
}

// an upper bound of the grid (the per-kernel grid is one resident wave, at
// most num_sms * 8 CTAs: the reduction partials hold MAXGRID)
int stencil3d_grid(int nx, int ny, int nz) {
    const long long work = stencil3d_work(nx, ny, nz), cap = (long long)num_sms() * 8;
    return (int)(work < cap ? work : cap);
}

template <typename T, int MODE, bool CROSS, bool HC>
static void launch3_one(bella_ws *ws, const StArgs3<T> &a, cudaStream_t s) {
    static int per_sm[64] = {0};            // resident CTAs per SM, queried once per device
    const size_t sm = smem3d_bytes<T>();
    const int dev = ws->device & 63;
    if (!per_sm[dev]) {
        cudaFuncSetAttribute(k_stencil3d<T, MODE, CROSS, HC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_stencil3d<T, MODE, CROSS, HC>, 256, sm) !=
                cudaSuccess || occ < 1)
            occ = 1;
        per_sm[dev] = occ < 8 ? occ : 8;
    }
    const long long work = stencil3d_work(ws->nx, ws->ny, ws->nz), wave = (long long)num_sms() * per_sm[dev];
    const int grid = (int)(work < wave ? work : wave);
    k_stencil3d<T, MODE, CROSS, HC><<<grid, 256, sm, s>>>(op3_of(ws, (T *)nullptr), a, ws->ks, ws->partials,
                                                         ws->counter);
}

template <typename T, int MODE>
static void launch3(bella_ws *ws, const StArgs3<T> &a, cudaStream_t s) {
    const int pk = MODE == M_PDIR ? PK_PDIR : MODE == M_SDIR ? PK_SDIR : MODE == M_RESID || MODE == M_RESX ? PK_RESID : -1;
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

void op3d_resid_df(bella_ws *ws, const double *x, const double *b, double *r, cudaStream_t s) {
    StArgs3<dfloat> a = {};
    a.x = reinterpret_cast<const dfloat *>(x);
    a.b = reinterpret_cast<const dfloat *>(b);
    a.y = reinterpret_cast<dfloat *>(r);
    launch3<dfloat, M_RESX>(ws, a, s);
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
