// bella_batch.cu -- the elliptic solves of an ensemble of 2D members with
// uneven grids in one persistent launch (sm_103a).
//
// Every member is the reference's solve (second_projection.py:205-230):
// scipy's BiCGStab on the Jacobi-scaled 9-point system, x0 = 0, FP64, stop at
// ||r|| <= max(tol*||b||, atol) with the scipy 1.7 legacy exit ||b|| <= tol.
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
#include <mutex>
#include <string>
#include <vector>

#include "bella_internal.cuh"

namespace bella {

struct BMember {
    Op2D<double> op;
    int cross, has_hc;
    double *x, *r, *rh, *p[2], *v[2], *t;
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

struct BArgs {
    const BMember *mem;
    BState *st;
    BCtl *ctl;
    double *partA, *partB, *partC;   // per-tile partials: P3 (2), P1 (1), P2 (3)
    int nmem, ntiles;
    double tol, atol_user;
    int maxiter;
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

__device__ MScal scal_p1(const BArgs &A, int m, int k) {
    const BMember &M = A.mem[m];
    const BState *S = &A.st[m];
    MScal c = {};
    double tot[2];
    member_totals<2>(A.partA, M.tile0, M.ntiles, tot);
    c.rho = tot[0];
    c.rr = tot[1];
    c.status = BELLA_MAXITER;
    if (k == 0) {
        c.bnorm = sqrt(c.rr);
        c.atol = A.tol * c.bnorm;
        if (A.atol_user > c.atol) c.atol = A.atol_user;
        if (!isfinite(c.rr)) { c.status = BELLA_NONFINITE; return c; }
        if (c.bnorm == 0.0 || c.bnorm <= A.tol) { c.status = BELLA_OK; return c; }   // scipy 1.7 legacy exit
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

__device__ MScal scal_p2(const BArgs &A, int m, int k) {
    const BMember &M = A.mem[m];
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

__device__ MScal scal_p3(const BArgs &A, int m, int k) {
    const BMember &M = A.mem[m];
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
template <int TXB, int TYB, int MODE>
__device__ void stencil_tile(const BMember &M, int lt, const MScal &c, int k, double *part,
                             double *su, double *sfx, double *sfy) {
    const Op2D<double> &op = M.op;
    const int nx = op.nx, ny = op.ny;
    const int tyi = lt / M.tilesx, txi = lt - tyi * M.tilesx;
    const int j0 = tyi * TYB, i0 = txi * TXB;
    const int par = k & 1;
    const double *pold = M.p[par ^ 1], *vold = M.v[par ^ 1];
    double *pnew = M.p[par], *vnew = M.v[par];
    const bool first = (k == 0);
    for (int e = threadIdx.x; e < (TYB + 2) * (TXB + 2); e += blockDim.x) {
        const int la = e / (TXB + 2), lb = e - la * (TXB + 2);
        int gj = j0 - 1 + la, gi = i0 - 1 + lb;
        if (gj < 0) gj += ny - 1; else if (gj == ny) gj = 1;
        if (gi < 0) gi += nx - 1; else if (gi == nx) gi = 1;
        double u = 0.0;
        if (gj < ny && gi < nx) {
            const size_t g = (size_t)gj * nx + gi;
            const double rg = __ldcg(&M.r[g]);
            if (MODE == 1) {
                u = first ? rg : rg + c.beta * (__ldcg(&pold[g]) - c.omega * __ldcg(&vold[g]));
                const bool owner = (la >= 1 && la <= TYB && lb >= 1 && lb <= TXB && j0 - 1 + la < ny && i0 - 1 + lb < nx);
                if (owner) pnew[g] = u;
            } else {
                u = rg - c.alpha * __ldcg(&vnew[g]);
            }
        }
        su[e] = u;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < (TYB + 1) * (TXB + 1); e += blockDim.x) {
        const int la = e / (TXB + 1), lb = e - la * (TXB + 1);
        const int cj = j0 + la, ci = i0 + lb;
        double fx = 0.0, fy = 0.0;
        if (cj <= ny && ci <= nx) {
            const size_t cc = (size_t)cj * (nx + 1) + ci;
            const double tl = su[la * (TXB + 2) + lb], tr = su[la * (TXB + 2) + lb + 1];
            const double bl = su[(la + 1) * (TXB + 2) + lb], br = su[(la + 1) * (TXB + 2) + lb + 1];
            const double gx = 0.5 * ((tr - tl) + (br - bl));
            const double gy = 0.5 * ((bl - tl) + (br - tr));
            fx = op.axx[cc] * gx;
            fy = op.ayy[cc] * gy;
            if (M.cross) {
                fx += op.axy[cc] * gy;
                fy += op.ayx[cc] * gx;
            }
        }
        sfx[e] = fx;
        sfy[e] = fy;
    }
    __syncthreads();
    double acc[3] = {0.0, 0.0, 0.0};
    for (int e = threadIdx.x; e < TYB * TXB; e += blockDim.x) {
        const int la = e / TXB, lb = e - la * TXB;
        const int gj = j0 + la, gi = i0 + lb;
        if (gj < ny && gi < nx) {
            const size_t g = (size_t)gj * nx + gi;
            const double u = su[(la + 1) * (TXB + 2) + lb + 1];
            const int W = TXB + 1;
            double s = ((sfx[la * W + lb + 1] + sfx[(la + 1) * W + lb + 1]) - (sfx[la * W + lb] + sfx[(la + 1) * W + lb])) +
                       ((sfy[(la + 1) * W + lb] + sfy[(la + 1) * W + lb + 1]) - (sfy[la * W + lb] + sfy[la * W + lb + 1]));
            if (M.has_hc) s += op.hc[g] * u;
            const double y = s * op.dinv[g];
            if (MODE == 1) {
                acc[0] += __ldcg(&M.rh[g]) * y;
                vnew[g] = y;
            } else {
                acc[0] += y * u;
                acc[1] += y * y;
                acc[2] += u * u;
                M.t[g] = y;
            }
        }
    }
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
template <int TXB, int TYB>
__device__ void update_tile(const BMember &M, int lt, const MScal &c, int k, const double *b, double *part) {
    const int nx = M.op.nx, ny = M.op.ny;
    const int tyi = lt / M.tilesx, txi = lt - tyi * M.tilesx;
    const int j0 = tyi * TYB, i0 = txi * TXB;
    double acc[2] = {0.0, 0.0};
    const int par = k & 1;
    for (int e = threadIdx.x; e < TYB * TXB; e += blockDim.x) {
        const int la = e / TXB, lb = e - la * TXB;
        const int gj = j0 + la, gi = i0 + lb;
        if (gj >= ny || gi >= nx) continue;
        const size_t g = (size_t)gj * nx + gi;
        if (k < 0) {
            const double bg = b[g];
            M.r[g] = bg;
            M.rh[g] = bg;
            M.x[g] = 0.0;
            acc[0] += bg * bg;
            acc[1] += bg * bg;
        } else {
            const double sg = __ldcg(&M.r[g]) - c.alpha * __ldcg(&M.v[par][g]);
            M.x[g] = M.x[g] + c.alpha * __ldcg(&M.p[par][g]) + c.omega * sg;
            const double rg = sg - c.omega * __ldcg(&M.t[g]);
            M.r[g] = rg;
            acc[0] += __ldcg(&M.rh[g]) * rg;
            acc[1] += rg * rg;
        }
    }
    __shared__ double red[32 * NQ];
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        part[(size_t)(M.tile0 + lt) * 2 + 0] = acc[0];
        part[(size_t)(M.tile0 + lt) * 2 + 1] = acc[1];
    }
    __syncthreads();
}

__device__ int member_of(const BArgs &A, int tile) {
    int lo = 0, hi = A.nmem - 1;   // members are in tile order
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.mem[mid].tile0 <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int TXB, int TYB>
__global__ void __launch_bounds__(256)
k_batch_bicgstab(BArgs A, const double *const *bptr) {
    __shared__ double su[(TYB + 2) * (TXB + 2)];
    __shared__ double sfx[(TYB + 1) * (TXB + 1)];
    __shared__ double sfy[(TYB + 1) * (TXB + 1)];
    // contiguous tile chunk of this block (consecutive tiles mostly share a member)
    const int t_begin = (int)((long long)A.ntiles * blockIdx.x / gridDim.x);
    const int t_end = (int)((long long)A.ntiles * (blockIdx.x + 1) / gridDim.x);
    // init: r = r^ = b, x = 0, <b, b>
    for (int t = t_begin; t < t_end; ++t) {
        const int m = member_of(A, t);
        MScal none = {};
        update_tile<TXB, TYB>(A.mem[m], t - A.mem[m].tile0, none, -1, bptr[m], A.partA);
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
                if (c.active) stencil_tile<TXB, TYB, 1>(A.mem[m], t - A.mem[m].tile0, c, k, A.partB, su, sfx, sfy);
            }
        }
        if (!grid_barrier(A.ctl)) return;
        if (__ldcg(&A.ctl->active[k & 1]) == 0) {
            if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl->iters = k;
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
                if (c.active) stencil_tile<TXB, TYB, 2>(A.mem[m], t - A.mem[m].tile0, c, k, A.partC, su, sfx, sfy);
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
                if (c.active) update_tile<TXB, TYB>(A.mem[m], t - A.mem[m].tile0, c, k, nullptr, A.partA);
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

typedef void (*BKernel)(BArgs, const double *const *);

static BKernel kernel_of(int tx, int ty) {
    if (tx == 64 && ty == 16) return k_batch_bicgstab<64, 16>;
    if (tx == 64 && ty == 8) return k_batch_bicgstab<64, 8>;
    if (tx == 32 && ty == 16) return k_batch_bicgstab<32, 16>;
    return k_batch_bicgstab<32, 8>;
}

struct BatchCtx {
    int device = -1;
    BMember *mem = nullptr;
    BState *st = nullptr;
    BCtl *ctl = nullptr;
    double *part = nullptr;
    const double **bptr = nullptr;
    size_t mem_cap = 0, part_cap = 0;
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
        if (cudaMalloc(&c.mem, nmem * sizeof(BMember)) != cudaSuccess ||
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

// one launch with configuration cfg; fills per-member results
static int batch_run(BatchCtx &c, bella_ws *const *ws, int nmem, const double *const *b, double *const *x,
                     const bella_solve_opts &o, int cfg, cudaStream_t s, std::vector<BState> *out, int *iters) {
    const BConfig K = kConfigs[cfg];
    std::vector<BMember> hm(nmem);
    int ntiles = 0;
    for (int m = 0; m < nmem; ++m) {
        bella_ws *w = ws[m];
        const size_t nc = (size_t)(w->nx + 1) * (w->ny + 1);
        BMember &M = hm[m];
        M.op.nx = w->nx; M.op.ny = w->ny;
        M.op.axx = w->a64; M.op.ayy = w->a64 + nc; M.op.axy = w->a64 + 2 * nc; M.op.ayx = w->a64 + 3 * nc;
        M.op.dinv = w->dinv64; M.op.hc = w->hc64;
        M.cross = w->cross; M.has_hc = w->has_hc;
        M.x = x[m]; M.r = w->r64k; M.rh = w->rh64;
        M.p[0] = w->p64[0]; M.p[1] = w->p64[1]; M.v[0] = w->v64[0]; M.v[1] = w->v64[1]; M.t = w->t64;
        M.tilesx = (w->nx + K.tx - 1) / K.tx;
        M.ntiles = M.tilesx * ((w->ny + K.ty - 1) / K.ty);
        M.tile0 = ntiles;
        ntiles += M.ntiles;
    }
    int rc = ctx_reserve(c, nmem, ntiles);
    if (rc != BELLA_OK) return rc;
    if (cudaMemcpyAsync(c.mem, hm.data(), nmem * sizeof(BMember), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(c.bptr, b, nmem * sizeof(double *), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(c.st, 0, nmem * sizeof(BState), s) != cudaSuccess ||
        cudaMemsetAsync(c.ctl, 0, sizeof(BCtl), s) != cudaSuccess)
        return BELLA_ECUDA;
    BArgs A;
    A.mem = c.mem; A.st = c.st; A.ctl = c.ctl;
    A.partA = c.part; A.partB = c.part + (size_t)ntiles * 2; A.partC = c.part + (size_t)ntiles * 3;
    A.nmem = nmem; A.ntiles = ntiles;
    A.tol = o.tol; A.atol_user = o.atol; A.maxiter = o.maxiter;
    BKernel kern = kernel_of(K.tx, K.ty);
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

static int check_members(bella_ws *const *ws, int nmem, const double *const *b, double *const *x) {
    if (!ws || !b || !x || nmem < 1) return BELLA_EINVAL;
    for (int m = 0; m < nmem; ++m) {
        if (!ws[m] || !b[m] || !x[m]) return BELLA_EINVAL;
        if (ws[m]->ndim != 2) return BELLA_ENOOP;
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
                         int probe_iters, int *choice, double *ms, void *stream) {
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
            rc = batch_run(c, ws, nmembers, b, x, o, cfg, s, nullptr, nullptr);
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
    const std::string sig = signature(ws, nmembers);
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
    int cfg = config;
    if (cfg < 0) {
        cfg = 0;
        const std::string sig = signature(ws, nmembers);
        for (auto &p : c.tuned)
            if (p.first == sig) cfg = p.second;
    }
    std::vector<BState> res;
    int iters = 0;
    rc = batch_run(c, ws, nmembers, b, x, o, cfg, s, &res, &iters);
    if (rc != BELLA_OK) return rc;
    // true FP64 residuals of all members, one synchronisation
    for (int m = 0; m < nmembers; ++m) op2d_resid(ws[m], 0, x[m], b[m], ws[m]->r64, s);
    std::vector<KState> ks(nmembers);
    for (int m = 0; m < nmembers; ++m)
        if (cudaMemcpyAsync(&ks[m], ws[m]->ks, sizeof(KState), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return BELLA_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return BELLA_ECUDA;
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int status = BELLA_OK;
    for (int m = 0; m < nmembers; ++m) {
        const BState &S = res[m];
        const int st_m = S.done ? S.status : BELLA_MAXITER;
        if (status == BELLA_OK && st_m != BELLA_OK) status = st_m;
        if (stats) {
            bella_solve_stats &q = stats[m];
            memset(&q, 0, sizeof(q));
            q.status = st_m;
            q.iterations = S.iter;
            q.matvecs = 2 * S.iter;
            q.bnorm = S.bnorm;
            const double rn = sqrt(ks[m].dot_aux2);
            q.relres = S.bnorm > 0 ? rn / S.bnorm : rn;
            q.seconds = secs;
            q.detail = S.detail;
            q.outer = cfg;
        }
    }
    (void)iters;
    return status;
}

}  // extern "C"
