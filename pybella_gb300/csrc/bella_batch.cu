// bella_batch.cu -- the elliptic solves of an ensemble of 2D members with
// uneven grids in one persistent launch (sm_103a).
//
// Every member is the reference's solve (second_projection.py:205-230):
// scipy's BiCGStab on the Jacobi-scaled 9-point system, x0 = 0, stop at
// ||r|| <= max(tol*||b||, atol) with the scipy 1.7 legacy exit ||b|| <= tol.
// Arithmetic: FP64, or double-float on the FP32 pipe (the default: GB300's
// FP64 pipe bounds the FP64 kernel); a double-float member whose FP64 true
// residual misses the tolerance is refined (FP64 residual, batched correction
// solve, FP64 update) by the host driver.
// Each member's operator and Krylov vectors live in its own workspace (set
// up by bella_op2d_set); one cooperative kernel walks the tiles of all
// members through the three phases of every iteration:
//   P1  p = r + beta (p - omega v) on the fly, v = A p, <r^, v>
//   P2  s = r - alpha v on the fly,  t = A s,  <t,s>, <t,t>, <s,s>
//   P3  x += alpha p + omega s,  r = s - omega t,  <r^, r>, ||r||^2
// separated by a grid barrier.  Inner products are per-tile partial sums
// reduced in tile order for each member, so every block derives a member's
// scalars (alpha, beta, omega, the stop tests) identically; one designated
// block per member records them.  A member that stops drops out; the launch
// ends when no member is active.  Tile shape and CTAs per SM come from the
// autotuner below (bella_batch_autotune).
#include <chrono>
#include <cstring>
#include <type_traits>
#include <mutex>
#include <string>
#include <vector>

#include "bella_internal.cuh"

namespace bella {

__global__ void k_dot64(long long n, const double *a, const double *b, KState *ks, double *partials,
                        unsigned *counter);

template <typename T> struct Num;
template <> struct Num<double> {
    static __device__ __forceinline__ double ld(const double *p) { return __ldcg(p); }
    static __device__ __forceinline__ double from(double d) { return d; }
    static __device__ __forceinline__ double to(double v) { return v; }
};
template <> struct Num<dfloat> {
    static __device__ __forceinline__ dfloat ld(const dfloat *p) {
        const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
        return dfloat(v.x, v.y);
    }
    static __device__ __forceinline__ dfloat from(double d) { return dfloat(d); }
    static __device__ __forceinline__ double to(dfloat v) { return v.to_double(); }
};

template <typename T>
struct BMember {
    Op2D<T> op;
    int cross, has_hc;
    T *x, *r, *rh, *p[2], *v[2], *t;
    double *xout;              // FP64 solution (== x for FP64 members)
    double rtol;               // relative tolerance of this member (||r|| <= rtol ||b||, or atol)
    int tile0, tilesx, ntiles;
};

struct BState {
    double rho[2], alpha[2], omega[2];
    double rho0, atol, bnorm;
    int iter, done, status, detail;
    int early;                 // ||s|| met the tolerance in P3 (stops at the next P1)
};

struct BCtl {
    unsigned count;            // barrier arrivals
    unsigned gen;              // barrier generation
    int err;                   // 1: a barrier wait gave up
    int active[2];             // members still iterating (by iteration parity)
    int iters;                 // iterations run by the launch
};

template <typename T>
struct BArgs {
    const BMember<T> *mem;
    BState *st;
    BCtl *ctl;
    double *partA, *partB, *partC;   // per-tile partials: P3 (2), P1 (1), P2 (3)
    int nmem, ntiles;
    double tol, atol_user;
    int maxiter;
    int legacy;                      // scipy 1.7 legacy exit ||b|| <= tol (off for refinement solves)
};

constexpr long long BARRIER_SPIN_LIMIT = 1LL << 26;   // about a few seconds with the back-off

// Grid barrier for a cooperative launch (all CTAs co-resident).  The wait is
// bounded: after BARRIER_SPIN_LIMIT polls it records an error and returns
// false, and the caller leaves the kernel.
__device__ bool grid_barrier(BCtl *ctl) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned *vgen = &ctl->gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->count, 1u);
        if (arrived == gridDim.x - 1) {
            ctl->count = 0;
            __threadfence();
            atomicAdd(&ctl->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (++spins > BARRIER_SPIN_LIMIT || *(volatile int *)&ctl->err) {
                    atomicExch(&ctl->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// member totals of Q partials (tile order, deterministic); valid in every thread
template <int Q>
__device__ void member_totals(const double *part, int tile0, int ntiles, double (&tot)[Q]) {
    __shared__ double red[32 * NQ];
    __shared__ double out[NQ];
    double v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = 0.0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
#pragma unroll
        for (int q = 0; q < Q; ++q) v[q] += __ldcg(&part[(size_t)(tile0 + t) * Q + q]);
    }
    block_sum<Q>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) out[q] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) tot[q] = out[q];
    __syncthreads();
}

// a flag that another block may be writing in this phase, read once per block so
// that every thread of the block takes the same path
__device__ int uniform_flag(const int *p) {
    __shared__ int v;
    __syncthreads();
    if (threadIdx.x == 0) v = __ldcg(p);
    __syncthreads();
    return v;
}

// scalars of a member for one phase, derived identically by every block
struct MScal {
    int active;        // member iterates in this phase
    int status, detail;
    double alpha, beta, omega, rho, rr, atol, bnorm;
    int early;
};

template <typename T>
__device__ MScal scal_p1(const BArgs<T> &A, int m, int k) {
    const BMember<T> &M = A.mem[m];
    const BState *S = &A.st[m];
    MScal c = {};
    double tot[2];
    member_totals<2>(A.partA, M.tile0, M.ntiles, tot);
    c.rho = tot[0];
    c.rr = tot[1];
    c.status = BELLA_MAXITER;
    if (k == 0) {
        c.bnorm = sqrt(c.rr);
        c.atol = M.rtol * c.bnorm;
        if (A.atol_user > c.atol) c.atol = A.atol_user;
        if (!isfinite(c.rr)) { c.status = BELLA_NONFINITE; return c; }
        if (c.bnorm == 0.0 || (A.legacy && c.bnorm <= A.tol)) { c.status = BELLA_OK; return c; }   // scipy 1.7 legacy exit
        if (A.maxiter <= 0) return c;
        c.active = 1;
        c.beta = 0.0;
        c.omega = 1.0;
        return c;
    }
    if (uniform_flag(&S->done)) { c.status = __ldcg(&S->status); return c; }
    if (__ldcg(&S->early)) { c.status = BELLA_OK; return c; }   // written in P3, stable here
    c.atol = __ldcg(&S->atol);
    const double rho_prev = __ldcg(&S->rho[(k - 1) & 1]);
    const double alpha = __ldcg(&S->alpha[(k - 1) & 1]), omega = __ldcg(&S->omega[(k - 1) & 1]);
    const double rho0 = __ldcg(&S->rho0);
    const double eps2 = 4.930380657631324e-32;
    if (!isfinite(c.rr) || !isfinite(c.rho)) { c.status = BELLA_NONFINITE; return c; }
    if (sqrt(c.rr) <= c.atol) { c.status = BELLA_OK; return c; }
    if (k >= A.maxiter) { c.status = BELLA_MAXITER; return c; }
    if (fabs(c.rho) < eps2 * rho0) { c.status = BELLA_BREAKDOWN; c.detail = 1; return c; }
    if (fabs(omega) < eps2) { c.status = BELLA_BREAKDOWN; c.detail = 2; return c; }
    c.active = 1;
    c.beta = (c.rho / rho_prev) * (alpha / omega);
    c.omega = omega;
    return c;
}

template <typename T>
__device__ MScal scal_p2(const BArgs<T> &A, int m, int k) {
    const BMember<T> &M = A.mem[m];
    const BState *S = &A.st[m];
    MScal c = {};
    if (uniform_flag(&S->done)) return c;
    double tot[1];
    member_totals<1>(A.partB, M.tile0, M.ntiles, tot);
    const double rho = __ldcg(&S->rho[k & 1]);
    if (!isfinite(tot[0])) { c.status = BELLA_NONFINITE; return c; }
    if (tot[0] == 0.0) { c.status = BELLA_BREAKDOWN; c.detail = 3; return c; }
    c.active = 1;
    c.alpha = rho / tot[0];
    return c;
}

template <typename T>
__device__ MScal scal_p3(const BArgs<T> &A, int m, int k) {
    const BMember<T> &M = A.mem[m];
    const BState *S = &A.st[m];
    MScal c = {};
    if (uniform_flag(&S->done)) return c;
    double tot[3];
    member_totals<3>(A.partC, M.tile0, M.ntiles, tot);
    c.alpha = __ldcg(&S->alpha[k & 1]);
    c.atol = __ldcg(&S->atol);
    const double ts = tot[0], tt = tot[1], ss = tot[2];
    if (!isfinite(ss) || !isfinite(ts) || !isfinite(tt)) { c.status = BELLA_NONFINITE; return c; }
    c.active = 1;
    if (sqrt(ss) <= c.atol) { c.early = 1; c.omega = 0.0; return c; }
    if (!(tt > 0.0)) { c.active = 0; c.status = BELLA_BREAKDOWN; c.detail = 4; return c; }
    c.omega = ts / tt;
    return c;
}

// one tile of P1 (MODE 1) or P2 (MODE 2): stage u with halo, cell fluxes, node outputs
template <typename T, int TXB, int TYB, int MODE>
__device__ void stencil_tile(const BMember<T> &M, int lt, const MScal &c, int k, double *part,
                             T *su, T *sfx, T *sfy) {
    using AccT = typename Acc<T>::type;
    const Op2D<T> &op = M.op;
    const int nx = op.nx, ny = op.ny;
    const int tyi = lt / M.tilesx, txi = lt - tyi * M.tilesx;
    const int j0 = tyi * TYB, i0 = txi * TXB;
    const int par = k & 1;
    const T *pold = M.p[par ^ 1], *vold = M.v[par ^ 1];
    T *pnew = M.p[par], *vnew = M.v[par];
    const bool first = (k == 0);
    const T beta = Num<T>::from(c.beta), omega = Num<T>::from(c.omega), alpha = Num<T>::from(c.alpha);
    const T zero = Num<T>::from(0.0);
    for (int e = threadIdx.x; e < (TYB + 2) * (TXB + 2); e += blockDim.x) {
        const int la = e / (TXB + 2), lb = e - la * (TXB + 2);
        int gj = j0 - 1 + la, gi = i0 - 1 + lb;
        if (gj < 0) gj += ny - 1; else if (gj == ny) gj = 1;
        if (gi < 0) gi += nx - 1; else if (gi == nx) gi = 1;
        T u = zero;
        if (gj < ny && gi < nx) {
            const size_t g = (size_t)gj * nx + gi;
            const T rg = Num<T>::ld(&M.r[g]);
            if (MODE == 1) {
                u = first ? rg : rg + beta * (Num<T>::ld(&pold[g]) - omega * Num<T>::ld(&vold[g]));
                const bool owner = (la >= 1 && la <= TYB && lb >= 1 && lb <= TXB && j0 - 1 + la < ny && i0 - 1 + lb < nx);
                if (owner) pnew[g] = u;
            } else {
                u = rg - alpha * Num<T>::ld(&vnew[g]);
            }
        }
        su[e] = u;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < (TYB + 1) * (TXB + 1); e += blockDim.x) {
        const int la = e / (TXB + 1), lb = e - la * (TXB + 1);
        const int cj = j0 + la, ci = i0 + lb;
        T fx = zero, fy = zero;
        if (cj <= ny && ci <= nx) {
            const size_t cc = (size_t)cj * (nx + 1) + ci;
            const T tl = su[la * (TXB + 2) + lb], tr = su[la * (TXB + 2) + lb + 1];
            const T bl = su[(la + 1) * (TXB + 2) + lb], br = su[(la + 1) * (TXB + 2) + lb + 1];
            const T d1 = br - tl, d2 = tr - bl;     // diagonal differences (bella_op2d.cu)
            const T gx = half_of(d1 + d2);
            const T gy = half_of(d1 - d2);
            fx = op.axx[cc] * gx;
            fy = op.ayy[cc] * gy;
            if (M.cross) {
                fx += op.axy[cc] * gy;
                fy += op.ayx[cc] * gx;
            }
        }
        sfx[e] = fx + fy;   // P
        sfy[e] = fx - fy;   // M
    }
    __syncthreads();
    AccT a0, a1, a2;
    a0.zero(); a1.zero(); a2.zero();
    for (int e = threadIdx.x; e < TYB * TXB; e += blockDim.x) {
        const int la = e / TXB, lb = e - la * TXB;
        const int gj = j0 + la, gi = i0 + lb;
        if (gj < ny && gi < nx) {
            const size_t g = (size_t)gj * nx + gi;
            const T u = su[(la + 1) * (TXB + 2) + lb + 1];
            const int W = TXB + 1;
            T s = (sfy[la * W + lb + 1] - sfy[(la + 1) * W + lb]) + (sfx[(la + 1) * W + lb + 1] - sfx[la * W + lb]);
            if (M.has_hc) s += op.hc[g] * u;
            const T y = s * op.dinv[g];
            if (MODE == 1) {
                a0.add_prod(Num<T>::ld(&M.rh[g]), y);
                vnew[g] = y;
            } else {
                a0.add_prod(y, u);
                a1.add_prod(y, y);
                a2.add_prod(u, u);
                M.t[g] = y;
            }
        }
    }
    double acc[3] = {a0.value(), a1.value(), a2.value()};
    __shared__ double red[32 * NQ];
    if (MODE == 1) {
        double v1[1] = {acc[0]};
        block_sum<1>(v1, red);
        if (threadIdx.x == 0) part[(size_t)(M.tile0 + lt)] = v1[0];
    } else {
        block_sum<3>(acc, red);
        if (threadIdx.x == 0) {
            part[(size_t)(M.tile0 + lt) * 3 + 0] = acc[0];
            part[(size_t)(M.tile0 + lt) * 3 + 1] = acc[1];
            part[(size_t)(M.tile0 + lt) * 3 + 2] = acc[2];
        }
    }
    __syncthreads();
}

// P3 on one tile (pointwise); also the initial r = b, r^ = b, x = 0 (k < 0)
template <typename T, int TXB, int TYB>
__device__ void update_tile(const BMember<T> &M, int lt, const MScal &c, int k, const double *b, double *part) {
    using AccT = typename Acc<T>::type;
    const int nx = M.op.nx, ny = M.op.ny;
    const int tyi = lt / M.tilesx, txi = lt - tyi * M.tilesx;
    const int j0 = tyi * TYB, i0 = txi * TXB;
    AccT a0, a1;
    a0.zero(); a1.zero();
    const int par = k & 1;
    const T alpha = Num<T>::from(c.alpha), omega = Num<T>::from(c.omega);
    for (int e = threadIdx.x; e < TYB * TXB; e += blockDim.x) {
        const int la = e / TXB, lb = e - la * TXB;
        const int gj = j0 + la, gi = i0 + lb;
        if (gj >= ny || gi >= nx) continue;
        const size_t g = (size_t)gj * nx + gi;
        if (k < 0) {
            const T bg = Num<T>::from(b[g]);
            M.r[g] = bg;
            M.rh[g] = bg;
            M.x[g] = Num<T>::from(0.0);
            a0.add_prod(bg, bg);
            a1.add_prod(bg, bg);
        } else {
            const T sg = Num<T>::ld(&M.r[g]) - alpha * Num<T>::ld(&M.v[par][g]);
            M.x[g] = (M.x[g] + alpha * Num<T>::ld(&M.p[par][g])) + omega * sg;
            const T rg = sg - omega * Num<T>::ld(&M.t[g]);
            M.r[g] = rg;
            a0.add_prod(Num<T>::ld(&M.rh[g]), rg);
            a1.add_prod(rg, rg);
        }
    }
    double acc[2] = {a0.value(), a1.value()};
    __shared__ double red[32 * NQ];
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        part[(size_t)(M.tile0 + lt) * 2 + 0] = acc[0];
        part[(size_t)(M.tile0 + lt) * 2 + 1] = acc[1];
    }
    __syncthreads();
}

template <typename T>
__device__ int member_of(const BArgs<T> &A, int tile) {
    int lo = 0, hi = A.nmem - 1;   // members are in tile order
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.mem[mid].tile0 <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// FP64 solution of a double-float member (tiles of this block's chunk)
template <typename T, int TXB, int TYB>
__device__ void export_x(const BArgs<T> &A, int t_begin, int t_end) {
    for (int t = t_begin; t < t_end; ++t) {
        const int m = member_of(A, t);
        const BMember<T> &M = A.mem[m];
        const int lt = t - M.tile0;
        const int tyi = lt / M.tilesx, txi = lt - tyi * M.tilesx;
        for (int e = threadIdx.x; e < TYB * TXB; e += blockDim.x) {
            const int gj = tyi * TYB + e / TXB, gi = txi * TXB + e % TXB;
            if (gj >= M.op.ny || gi >= M.op.nx) continue;
            const size_t g = (size_t)gj * M.op.nx + gi;
            M.xout[g] = Num<T>::to(M.x[g]);
        }
    }
}

template <typename T, int TXB, int TYB>
__global__ void __launch_bounds__(256)
k_batch_bicgstab(BArgs<T> A, const double *const *bptr) {
    __shared__ T su[(TYB + 2) * (TXB + 2)];
    __shared__ T sfx[(TYB + 1) * (TXB + 1)];
    __shared__ T sfy[(TYB + 1) * (TXB + 1)];
    // contiguous tile chunk of this block (consecutive tiles mostly share a member)
    const int t_begin = (int)((long long)A.ntiles * blockIdx.x / gridDim.x);
    const int t_end = (int)((long long)A.ntiles * (blockIdx.x + 1) / gridDim.x);
    // init: r = r^ = b, x = 0, <b, b>
    for (int t = t_begin; t < t_end; ++t) {
        const int m = member_of(A, t);
        MScal none = {};
        update_tile<T, TXB, TYB>(A.mem[m], t - A.mem[m].tile0, none, -1, bptr[m], A.partA);
    }
    if (!grid_barrier(A.ctl)) return;
    for (int k = 0;; ++k) {
        // ---- P1: stop tests and beta, p and v = A p, <r^, v>
        if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl->active[(k + 1) & 1] = 0;
        for (int m = blockIdx.x; m < A.nmem; m += gridDim.x) {     // designated block of member m
            const MScal c = scal_p1(A, m, k);
            if (threadIdx.x == 0) {
                BState *S = &A.st[m];
                if (k == 0) { S->atol = c.atol; S->bnorm = c.bnorm; S->rho0 = c.rho; S->iter = 0; S->done = 0; S->detail = 0; }
                if (c.active) {
                    S->rho[k & 1] = c.rho;
                    atomicAdd(&A.ctl->active[k & 1], 1);
                } else if (!S->done) {
                    S->done = 1;
                    S->status = c.status;
                    S->detail = c.detail;
                }
            }
        }
        {
            int cur = -1;
            MScal c = {};
            for (int t = t_begin; t < t_end; ++t) {
                const int m = member_of(A, t);
                if (m != cur) { c = scal_p1(A, m, k); cur = m; }
                if (c.active) stencil_tile<T, TXB, TYB, 1>(A.mem[m], t - A.mem[m].tile0, c, k, A.partB, su, sfx, sfy);
            }
        }
        if (!grid_barrier(A.ctl)) return;
        if (__ldcg(&A.ctl->active[k & 1]) == 0) {
            if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl->iters = k;
            if (!std::is_same<T, double>::value) export_x<T, TXB, TYB>(A, t_begin, t_end);
            return;
        }
        // ---- P2: alpha, s and t = A s, <t,s>, <t,t>, <s,s>
        for (int m = blockIdx.x; m < A.nmem; m += gridDim.x) {
            const MScal c = scal_p2(A, m, k);
            if (threadIdx.x == 0 && !__ldcg(&A.st[m].done)) {
                if (c.active) A.st[m].alpha[k & 1] = c.alpha;   // a member that stopped in P1 is done already
                else { A.st[m].done = 1; A.st[m].status = c.status; A.st[m].detail = c.detail; A.st[m].iter = k; }
            }
        }
        {
            int cur = -1;
            MScal c = {};
            for (int t = t_begin; t < t_end; ++t) {
                const int m = member_of(A, t);
                if (m != cur) { c = scal_p2(A, m, k); cur = m; }
                if (c.active) stencil_tile<T, TXB, TYB, 2>(A.mem[m], t - A.mem[m].tile0, c, k, A.partC, su, sfx, sfy);
            }
        }
        if (!grid_barrier(A.ctl)) return;
        // ---- P3: omega (early exit on ||s||), x and r, <r^, r>, ||r||^2
        for (int m = blockIdx.x; m < A.nmem; m += gridDim.x) {
            const MScal c = scal_p3(A, m, k);
            if (threadIdx.x == 0 && !__ldcg(&A.st[m].done)) {
                BState *S = &A.st[m];
                if (c.active) {
                    S->omega[k & 1] = c.omega;
                    S->iter = k + 1;
                    if (c.early) S->early = 1;   // every block still applies this P3 update
                } else {
                    S->done = 1; S->status = c.status; S->detail = c.detail; S->iter = k;
                }
            }
        }
        {
            int cur = -1;
            MScal c = {};
            for (int t = t_begin; t < t_end; ++t) {
                const int m = member_of(A, t);
                if (m != cur) { c = scal_p3(A, m, k); cur = m; }
                if (c.active) update_tile<T, TXB, TYB>(A.mem[m], t - A.mem[m].tile0, c, k, nullptr, A.partA);
            }
        }
        if (!grid_barrier(A.ctl)) return;
    }
}

// ---------------------------------------------------------------------------
// host side: launch configurations and the autotuner
// ---------------------------------------------------------------------------
struct BConfig { int tx, ty, per_sm; };
static const BConfig kConfigs[] = {{64, 16, 0}, {64, 8, 0}, {32, 16, 0}, {32, 8, 0}, {64, 8, 2}, {32, 8, 2}};
constexpr int NCONFIG = (int)(sizeof(kConfigs) / sizeof(kConfigs[0]));

template <typename T>
using BKernel = void (*)(BArgs<T>, const double *const *);

template <typename T>
static BKernel<T> kernel_of(int tx, int ty) {
    if (tx == 64 && ty == 16) return k_batch_bicgstab<T, 64, 16>;
    if (tx == 64 && ty == 8) return k_batch_bicgstab<T, 64, 8>;
    if (tx == 32 && ty == 16) return k_batch_bicgstab<T, 32, 16>;
    return k_batch_bicgstab<T, 32, 8>;
}

struct BatchCtx {
    int device = -1;
    void *mem = nullptr;      // BMember<T>[] (same size for both arithmetic types)
    BState *st = nullptr;
    BCtl *ctl = nullptr;
    double *part = nullptr;
    const double **bptr = nullptr;
    size_t mem_cap = 0, part_cap = 0;
    double *save = nullptr;   // a member's iterate kept while it is finished alone
    long long save_cap = 0;
    // autotuned choice per member-size signature
    std::vector<std::pair<std::string, int>> tuned;
    std::string err;
};

static std::mutex g_batch_mu;
static BatchCtx g_batch[64];

static int ctx_reserve(BatchCtx &c, int nmem, int ntiles) {
    if ((size_t)nmem > c.mem_cap) {
        cudaFree(c.mem); cudaFree(c.st); cudaFree(c.bptr);
        c.mem = nullptr; c.st = nullptr; c.bptr = nullptr; c.mem_cap = 0;
        if (cudaMalloc(&c.mem, nmem * sizeof(BMember<double>)) != cudaSuccess ||
            cudaMalloc(&c.st, nmem * sizeof(BState)) != cudaSuccess ||
            cudaMalloc((void **)&c.bptr, nmem * sizeof(double *)) != cudaSuccess)
            return BELLA_ECUDA;
        c.mem_cap = nmem;
    }
    if ((size_t)ntiles > c.part_cap) {
        cudaFree(c.part);
        c.part = nullptr; c.part_cap = 0;
        if (cudaMalloc(&c.part, (size_t)ntiles * 6 * sizeof(double)) != cudaSuccess) return BELLA_ECUDA;
        c.part_cap = ntiles;
    }
    if (!c.ctl && cudaMalloc(&c.ctl, sizeof(BCtl)) != cudaSuccess) return BELLA_ECUDA;
    return BELLA_OK;
}

static std::string signature(bella_ws *const *ws, int nmem) {
    std::string s;
    for (int m = 0; m < nmem; ++m) s += std::to_string(ws[m]->nx) + "x" + std::to_string(ws[m]->ny) + ";";
    return s;
}

template <typename T> static void member_vectors(BMember<T> &M, bella_ws *w, double *x);
template <> void member_vectors<double>(BMember<double> &M, bella_ws *w, double *x) {
    const size_t nc = (size_t)(w->nx + 1) * (w->ny + 1);
    M.op.axx = w->a64; M.op.ayy = w->a64 + nc; M.op.axy = w->a64 + 2 * nc; M.op.ayx = w->a64 + 3 * nc;
    M.op.dinv = w->dinv64; M.op.hc = w->hc64;
    M.x = x; M.xout = x; M.r = w->r64k; M.rh = w->rh64;
    M.p[0] = w->p64[0]; M.p[1] = w->p64[1]; M.v[0] = w->v64[0]; M.v[1] = w->v64[1]; M.t = w->t64;
}
template <> void member_vectors<dfloat>(BMember<dfloat> &M, bella_ws *w, double *x) {
    const size_t nc = (size_t)(w->nx + 1) * (w->ny + 1);
    M.op.axx = w->adf; M.op.ayy = w->adf + nc; M.op.axy = w->adf + 2 * nc; M.op.ayx = w->adf + 3 * nc;
    M.op.dinv = w->dinvdf; M.op.hc = w->hcdf;
    M.x = w->xdf; M.xout = x; M.r = w->rdf; M.rh = w->rhdf;
    M.p[0] = w->pdf[0]; M.p[1] = w->pdf[1]; M.v[0] = w->vdf[0]; M.v[1] = w->vdf[1]; M.t = w->tdf;
}

// one launch with configuration cfg; fills per-member results
template <typename T>
static int batch_run(BatchCtx &c, bella_ws *const *ws, int nmem, const double *const *b, double *const *x,
                     const bella_solve_opts &o, int cfg, cudaStream_t s, std::vector<BState> *out, int *iters,
                     int legacy, const double *rtol) {
    const BConfig K = kConfigs[cfg];
    std::vector<BMember<T>> hm(nmem);
    int ntiles = 0;
    for (int m = 0; m < nmem; ++m) {
        bella_ws *w = ws[m];
        BMember<T> &M = hm[m];
        M.op.nx = w->nx; M.op.ny = w->ny;
        member_vectors<T>(M, w, x[m]);
        M.cross = w->cross; M.has_hc = w->has_hc;
        M.rtol = rtol ? rtol[m] : o.tol;
        M.tilesx = (w->nx + K.tx - 1) / K.tx;
        M.ntiles = M.tilesx * ((w->ny + K.ty - 1) / K.ty);
        M.tile0 = ntiles;
        ntiles += M.ntiles;
    }
    int rc = ctx_reserve(c, nmem, ntiles);
    if (rc != BELLA_OK) return rc;
    if (cudaMemcpyAsync(c.mem, hm.data(), nmem * sizeof(BMember<T>), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(c.bptr, b, nmem * sizeof(double *), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(c.st, 0, nmem * sizeof(BState), s) != cudaSuccess ||
        cudaMemsetAsync(c.ctl, 0, sizeof(BCtl), s) != cudaSuccess)
        return BELLA_ECUDA;
    BArgs<T> A;
    A.mem = (const BMember<T> *)c.mem; A.st = c.st; A.ctl = c.ctl;
    A.partA = c.part; A.partB = c.part + (size_t)ntiles * 2; A.partC = c.part + (size_t)ntiles * 3;
    A.nmem = nmem; A.ntiles = ntiles;
    A.tol = o.tol; A.atol_user = o.atol; A.maxiter = o.maxiter;
    A.legacy = legacy;
    BKernel<T> kern = kernel_of<T>(K.tx, K.ty);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0) != cudaSuccess || per_sm < 1)
        return BELLA_ECUDA;
    if (K.per_sm > 0 && K.per_sm < per_sm) per_sm = K.per_sm;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ws[0]->device);
    int grid = per_sm * nsm;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    const double *const *bp = c.bptr;
    void *args[] = {&A, &bp};
    if (cudaLaunchCooperativeKernel((const void *)kern, grid, 256, args, 0, s) != cudaSuccess) return BELLA_ECUDA;
    if (out) {
        out->resize(nmem);
        BCtl hc;
        if (cudaMemcpyAsync(out->data(), c.st, nmem * sizeof(BState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(&hc, c.ctl, sizeof(BCtl), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return BELLA_ECUDA;
        if (hc.err) return BELLA_ECUDA;   // a grid barrier wait gave up (bounded spin)
        if (iters) *iters = hc.iters;
    }
    return BELLA_OK;
}

static int batch_run_prec(int prec, BatchCtx &c, bella_ws *const *ws, int nmem, const double *const *b,
                          double *const *x, const bella_solve_opts &o, int cfg, cudaStream_t s,
                          std::vector<BState> *out, int *iters, int legacy = 1, const double *rtol = nullptr) {
    if (prec == 0) return batch_run<double>(c, ws, nmem, b, x, o, cfg, s, out, iters, legacy, rtol);
    return batch_run<dfloat>(c, ws, nmem, b, x, o, cfg, s, out, iters, legacy, rtol);
}

// x += a d
__global__ void k_batch_axpy(long long n, double a, const double *d, double *x) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] += a * d[i];
}

// y = a x
__global__ void k_batch_scale(long long n, double a, const double *x, double *y) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = a * x[i];
}

// ||b_m|| of every member (one synchronisation)
static int member_norms(bella_ws *const *ws, int nmem, const double *const *b, cudaStream_t s, std::vector<double> &bn) {
    std::vector<KState> ks(nmem);
    for (int m = 0; m < nmem; ++m)
        k_dot64<<<ws[m]->grid_vec, VEC_BLOCK, 0, s>>>(ws[m]->n, b[m], b[m], ws[m]->ks, ws[m]->partials, ws[m]->counter);
    for (int m = 0; m < nmem; ++m)
        if (cudaMemcpyAsync(&ks[m], ws[m]->ks, sizeof(KState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return BELLA_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return BELLA_ECUDA;
    bn.resize(nmem);
    for (int m = 0; m < nmem; ++m) bn[m] = sqrt(ks[m].dot_aux);
    return BELLA_OK;
}

static int check_members(bella_ws *const *ws, int nmem, const double *const *b, double *const *x) {
    if (!ws || !b || !x || nmem < 1) return BELLA_EINVAL;
    for (int m = 0; m < nmem; ++m) {
        if (!ws[m] || !b[m] || !x[m]) return BELLA_EINVAL;
        if (ws[m]->ndim != 2) return BELLA_ENOOP;
        if (ws[m]->ymirror) return BELLA_EINVAL;     // the batched stencil wraps y (no LAMB_BDRY mirror)
        if (ws[m]->device != ws[0]->device) return BELLA_EINVAL;
    }
    return BELLA_OK;
}

}  // namespace bella

using namespace bella;

extern "C" {

// Autotuner: times every launch configuration on maxiter_probe iterations of
// the batch and keeps the fastest for this set of member sizes.  *choice
// (optional) receives its index; *ms (optional, NCONFIG entries) the times.
int bella_batch_autotune(bella_ws *const *ws, int nmembers, const double *const *b, double *const *x,
                         int precision, int probe_iters, int *choice, double *ms, void *stream) {
    const int prec = precision == 0 ? 0 : 2;
    int rc = check_members(ws, nmembers, b, x);
    if (rc != BELLA_OK) return rc;
    std::lock_guard<std::mutex> lk(g_batch_mu);
    const int dev = ws[0]->device;
    if (dev < 0 || dev >= 64) return BELLA_EINVAL;
    if (cudaSetDevice(dev) != cudaSuccess) return BELLA_ECUDA;
    BatchCtx &c = g_batch[dev];
    cudaStream_t s = (cudaStream_t)stream;
    bella_solve_opts o;
    bella_solve_opts_default(&o);
    o.tol = 0.0;
    o.maxiter = probe_iters > 0 ? probe_iters : 20;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = 0;
    float best_ms = 1e30f;
    for (int cfg = 0; cfg < NCONFIG; ++cfg) {
        float t = 0.f;
        for (int rep = 0; rep < 2; ++rep) {   // first run warms up
            cudaEventRecord(e0, s);
            rc = batch_run_prec(prec, c, ws, nmembers, b, x, o, cfg, s, nullptr, nullptr);
            if (rc != BELLA_OK) break;
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) { rc = BELLA_ECUDA; break; }
            cudaEventElapsedTime(&t, e0, e1);
        }
        if (rc != BELLA_OK) break;
        if (ms) ms[cfg] = t;
        if (t < best_ms) { best_ms = t; best = cfg; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != BELLA_OK) return rc;
    const std::string sig = signature(ws, nmembers) + (prec == 0 ? "fp64" : "df64");
    bool found = false;
    for (auto &p : c.tuned)
        if (p.first == sig) { p.second = best; found = true; }
    if (!found) c.tuned.emplace_back(sig, best);
    if (choice) *choice = best;
    return BELLA_OK;
}

int bella_batch_config_count(void) { return NCONFIG; }

int bella_batch_config(int index, int *tile_x, int *tile_y, int *ctas_per_sm) {
    if (index < 0 || index >= NCONFIG) return BELLA_EINVAL;
    if (tile_x) *tile_x = kConfigs[index].tx;
    if (tile_y) *tile_y = kConfigs[index].ty;
    if (ctas_per_sm) *ctas_per_sm = kConfigs[index].per_sm;
    return BELLA_OK;
}

// FP64 BiCGStab (scipy control flow, x0 = 0) for nmembers 2D systems in one
// persistent launch.  ws[m]: workspace with member m's operator
// (bella_op2d_set); b[m], x[m]: device FP64 vectors of its nx*ny nodes.
// opts: tol, atol, maxiter (shared); config < 0 takes the autotuned choice for
// these member sizes (the first configuration when none was tuned).
// stats[m] (optional): iterations, status, detail, bnorm and the true FP64
// relative residual.  Returns BELLA_OK when every member converged, else the
// first non-OK member status; BELLA_ECUDA if a grid barrier wait gave up.
int bella_bicgstab_batched(bella_ws *const *ws, int nmembers, const double *const *b, double *const *x,
                           const bella_solve_opts *opts, int config, bella_solve_stats *stats, void *stream) {
    int rc = check_members(ws, nmembers, b, x);
    if (rc != BELLA_OK) return rc;
    if (config >= NCONFIG) return BELLA_EINVAL;
    std::lock_guard<std::mutex> lk(g_batch_mu);
    const int dev = ws[0]->device;
    if (dev < 0 || dev >= 64) return BELLA_EINVAL;
    if (cudaSetDevice(dev) != cudaSuccess) return BELLA_ECUDA;
    BatchCtx &c = g_batch[dev];
    cudaStream_t s = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    bella_solve_opts o;
    if (opts) o = *opts; else bella_solve_opts_default(&o);
    if (!(o.tol >= 0.0) || o.maxiter < 0) return BELLA_EINVAL;
    const int prec = o.precision == 0 ? 0 : 2;
    int cfg = config;
    if (cfg < 0) {
        cfg = 0;
        const std::string sig = signature(ws, nmembers) + (prec == 0 ? "fp64" : "df64");
        for (auto &p : c.tuned)
            if (p.first == sig) cfg = p.second;
    }
    std::vector<int> status(nmembers, BELLA_OK), its(nmembers, 0), detail(nmembers, 0), rounds(nmembers, 0);
    std::vector<double> bnorm(nmembers, 0.0);
    std::vector<KState> ks(nmembers);
    if (prec == 0) {
        // FP64: the scipy path as it is
        std::vector<BState> res;
        int iters = 0;
        rc = batch_run_prec(prec, c, ws, nmembers, b, x, o, cfg, s, &res, &iters);
        if (rc != BELLA_OK) return rc;
        for (int m = 0; m < nmembers; ++m) {
            status[m] = res[m].done ? res[m].status : BELLA_MAXITER;
            its[m] = res[m].iter;
            detail[m] = res[m].detail;
            bnorm[m] = res[m].bnorm;
        }
    } else {
        // Double-float has the FP32 exponent range: every member solves its system
        // scaled to a unit right-hand side (BiCGStab is scale-invariant), with its
        // own relative tolerance; then x = ||b|| x'.  The scipy 1.7 legacy exit
        // uses the unscaled ||b||.
        rc = member_norms(ws, nmembers, b, s, bnorm);
        if (rc != BELLA_OK) return rc;
        std::vector<bella_ws *> sw;
        std::vector<const double *> sb;
        std::vector<double *> sx;
        std::vector<double> rt;
        std::vector<int> idx;
        for (int m = 0; m < nmembers; ++m) {
            if (!isfinite(bnorm[m])) { status[m] = BELLA_NONFINITE; continue; }
            if (bnorm[m] == 0.0 || bnorm[m] <= o.tol) {
                if (cudaMemsetAsync(x[m], 0, ws[m]->n * sizeof(double), s) != cudaSuccess) return BELLA_ECUDA;
                continue;
            }
            k_batch_scale<<<vec_grid(ws[m]->n), VEC_BLOCK, 0, s>>>(ws[m]->n, 1.0 / bnorm[m], b[m], ws[m]->r64);
            idx.push_back(m);
            sw.push_back(ws[m]);
            sb.push_back(ws[m]->r64);
            sx.push_back(x[m]);
            double r = o.tol;
            if (o.atol / bnorm[m] > r) r = o.atol / bnorm[m];
            rt.push_back(r);
        }
        bella_solve_opts oi = o;
        oi.atol = 0.0;
        if (!idx.empty()) {
            std::vector<BState> res;
            int iters = 0;
            rc = batch_run_prec(prec, c, sw.data(), (int)idx.size(), sb.data(), sx.data(), oi, cfg, s, &res, &iters, 0,
                                rt.data());
            if (rc != BELLA_OK) return rc;
            for (size_t q = 0; q < idx.size(); ++q) {
                const int m = idx[q];
                status[m] = res[q].done ? res[q].status : BELLA_MAXITER;
                its[m] = res[q].iter;
                detail[m] = res[q].detail;
                k_batch_scale<<<vec_grid(ws[m]->n), VEC_BLOCK, 0, s>>>(ws[m]->n, bnorm[m], x[m], x[m]);
            }
        }
    }
    // FP64 true residuals; double-float members that converged on the recursion
    // but miss the tolerance in FP64 are refined: d solves A d = r / ||r|| (x0 = 0)
    // in a batched launch of just those members, x += ||r|| d, up to 4 rounds
    for (int round = 0;; ++round) {
        for (int m = 0; m < nmembers; ++m) op2d_resid(ws[m], 0, x[m], b[m], ws[m]->r64, s);
        for (int m = 0; m < nmembers; ++m)
            if (cudaMemcpyAsync(&ks[m], ws[m]->ks, sizeof(KState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
                return BELLA_ECUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return BELLA_ECUDA;
        if (prec == 0 || round >= 4) break;
        std::vector<bella_ws *> sw;
        std::vector<const double *> sb;
        std::vector<double *> sx;
        std::vector<double> rt, rn;
        std::vector<int> idx;
        for (int m = 0; m < nmembers; ++m) {
            double target = o.tol * bnorm[m];
            if (o.atol > target) target = o.atol;
            const double r = sqrt(ks[m].dot_aux2);
            if (status[m] == BELLA_OK && isfinite(r) && r > target && r > 0.0) {
                k_batch_scale<<<vec_grid(ws[m]->n), VEC_BLOCK, 0, s>>>(ws[m]->n, 1.0 / r, ws[m]->r64, ws[m]->r64);
                idx.push_back(m);
                sw.push_back(ws[m]);
                sb.push_back(ws[m]->r64);
                sx.push_back(ws[m]->x64v);
                rt.push_back(0.5 * target / r);
                rn.push_back(r);
            }
        }
        if (idx.empty()) break;
        bella_solve_opts oi = o;
        oi.atol = 0.0;
        std::vector<BState> sub;
        int it2 = 0;
        rc = batch_run_prec(prec, c, sw.data(), (int)idx.size(), sb.data(), sx.data(), oi, cfg, s, &sub, &it2, 0,
                            rt.data());
        if (rc != BELLA_OK) return rc;
        for (size_t q = 0; q < idx.size(); ++q) {
            const int m = idx[q];
            k_batch_axpy<<<vec_grid(ws[m]->n), VEC_BLOCK, 0, s>>>(ws[m]->n, rn[q], ws[m]->x64v, x[m]);
            its[m] += sub[q].iter;
            rounds[m] += 1;
            if (!sub[q].done || sub[q].status != BELLA_OK) status[m] = sub[q].done ? sub[q].status : BELLA_MAXITER;
        }
    }
    // double-float members whose batched iteration broke down, or whose FP64 true
    // residual still misses the tolerance after the refinement rounds (the
    // double-float floor of a hard system), are finished one by one by the FP64
    // solve from their iterate, within the iteration budget left; the batched
    // iterate is kept unless that lowers its FP64 true residual.  Reported in
    // stats->fallback.
    std::vector<int> single(nmembers, 0);
    if (prec != 0) {
        bool any = false;
        for (int m = 0; m < nmembers; ++m) {
            double target = o.tol * bnorm[m];
            if (o.atol > target) target = o.atol;
            const double rm = sqrt(ks[m].dot_aux2);
            const bool missed = status[m] == BELLA_OK && isfinite(rm) && rm > target && !(bnorm[m] <= o.tol);
            if (!(status[m] == BELLA_BREAKDOWN || missed) || !isfinite(bnorm[m]) || !isfinite(rm) ||
                its[m] >= o.maxiter)
                continue;
            const long long nm_ = ws[m]->n;
            if (c.save_cap < nm_) {
                cudaFree(c.save);
                c.save = nullptr;
                c.save_cap = 0;
                if (cudaMalloc(&c.save, nm_ * sizeof(double)) != cudaSuccess) return BELLA_ECUDA;
                c.save_cap = nm_;
            }
            if (cudaMemcpyAsync(c.save, x[m], nm_ * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return BELLA_ECUDA;
            bella_solve_opts os = o;
            os.precision = 0;
            os.x0_zero = 0;
            os.maxiter = o.maxiter - its[m];
            bella_solve_stats fs;
            const int r = bella_bicgstab(ws[m], b[m], x[m], &os, &fs, stream);
            if (r < 0) return r;
            its[m] += fs.iterations;
            if (isfinite(fs.relres) && fs.relres * bnorm[m] < rm) {
                status[m] = fs.status;
                single[m] = 1;
            } else if (cudaMemcpyAsync(x[m], c.save, nm_ * sizeof(double), cudaMemcpyDeviceToDevice, s) !=
                       cudaSuccess) {
                return BELLA_ECUDA;
            }
            any = true;
        }
        if (any) {
            for (int m = 0; m < nmembers; ++m)
                if (single[m]) op2d_resid(ws[m], 0, x[m], b[m], ws[m]->r64, s);
            for (int m = 0; m < nmembers; ++m)
                if (single[m] && cudaMemcpyAsync(&ks[m], ws[m]->ks, sizeof(KState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
                    return BELLA_ECUDA;
            if (cudaStreamSynchronize(s) != cudaSuccess) return BELLA_ECUDA;
        }
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int worst = BELLA_OK;
    for (int m = 0; m < nmembers; ++m) {
        double target = o.tol * bnorm[m];
        if (o.atol > target) target = o.atol;
        const double rn = sqrt(ks[m].dot_aux2);
        int st_m = status[m];
        if (st_m == BELLA_OK && !(rn <= target) && !(bnorm[m] <= o.tol)) st_m = BELLA_MAXITER;   // never on the recursion alone
        if (!isfinite(rn)) st_m = BELLA_NONFINITE;
        if (worst == BELLA_OK && st_m != BELLA_OK) worst = st_m;
        if (stats) {
            bella_solve_stats &q = stats[m];
            memset(&q, 0, sizeof(q));
            q.status = st_m;
            q.iterations = its[m];
            q.matvecs = 2 * its[m];
            q.bnorm = bnorm[m];
            q.relres = bnorm[m] > 0 ? rn / bnorm[m] : rn;
            q.seconds = secs;
            q.detail = detail[m];
            q.outer = cfg;
            q.fallback = rounds[m] + (single[m] ? 256 : 0);   // FP64 refinement rounds; +256: finished alone
        }
    }
    return worst;
}

}  // extern "C"
