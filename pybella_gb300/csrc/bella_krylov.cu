// bella_krylov.cu -- streaming Krylov kernels, the BiCGStab / mixed-precision
// iterative-refinement driver and the C ABI of libbella_gb300.
//
// Solver contract: the reference's scipy call
//   p2, _ = scipy.sparse.linalg.bicgstab(lap, rhs_inner, tol=ud.tol,
//                                        maxiter=ud.max_iterations, callback=counter)
// (second_projection.py:230), with scipy 1.7 legacy `tol` semantics.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>

#include "bella_internal.cuh"

namespace bella {

static thread_local std::string g_err;

int set_err(int code, const char *what) {
    g_err = what;
    return code;
}

int cuda_check(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return BELLA_OK;
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return BELLA_ECUDA;
}

#define BELLA_CUDA(call)                                             \
    do {                                                             \
        int _rc = cuda_check((call), #call);                         \
        if (_rc != BELLA_OK) return _rc;                             \
    } while (0)

int num_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    std::atomic<int> *c = dev < 64 ? &cache[dev] : nullptr;
    int n = c ? c->load(std::memory_order_relaxed) : 0;
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    if (n > MAX_SMS) n = MAX_SMS;
    if (c) c->store(n, std::memory_order_relaxed);
    return n;
}

int vec_grid(long long n) {
    long long g = (n + VEC_BLOCK - 1) / VEC_BLOCK;
    const long long cap = (long long)num_sms() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// --------------------------------------------------------------------------
// vector kernels
// --------------------------------------------------------------------------
// x += alpha p + omega s,  r = s - omega t  (s = r - alpha v recomputed),
// with <r^, r> and ||r||^2 of the new residual.
template <typename T>
__global__ void __launch_bounds__(VEC_BLOCK)
k_update(long long n, T *x, const T *p0, const T *p1, T *r, const T *v0, const T *v1, const T *t,
         const T *rh, KState *ks, double *partials, unsigned *counter) {
    using AccT = typename Acc<T>::type;
    if (ks->done) return;
    const int par = ks->iter & 1;
    const T *p = par ? p0 : p1;   // p/v written by this iteration's PDIR kernel
    const T *v = par ? v0 : v1;
    const T alpha = (T)ks->alpha, omega = (T)ks->omega;
    const bool early = ks->early != 0;
    AccT a0, a1;
    a0.zero(); a1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const T pg = p[g];
        if (early) {
            x[g] += alpha * pg;
        } else {
            const T s = r[g] - alpha * v[g];
            x[g] += alpha * pg + omega * s;
            const T rn = s - omega * t[g];
            r[g] = rn;
            a0.add_prod(rh[g], rn);
            a1.add_prod(rn, rn);
        }
    }
    double vv[2] = {a0.value(), a1.value()}, tot[2];
    if (!grid_sum<2>(vv, partials, counter, tot)) return;
    if (threadIdx.x == 0) finalize_update(ks, tot[0], tot[1]);
}

void prof_begin(bella_ws *ws, int kind, cudaStream_t s) {
    if (!ws->prof) return;
    bella_ws::Prof &p = ws->profk[kind];
    if (p.pending == 256) prof_harvest(ws);
    cudaEventRecord(p.ev[2 * p.pending], s);
}

void prof_end(bella_ws *ws, int kind, cudaStream_t s) {
    if (!ws->prof) return;
    bella_ws::Prof &p = ws->profk[kind];
    cudaEventRecord(p.ev[2 * p.pending + 1], s);
    p.pending++;
}

void prof_harvest(bella_ws *ws) {
    if (!ws->prof) return;
    for (int k = 0; k < 4; ++k) {
        bella_ws::Prof &p = ws->profk[k];
        for (int i = 0; i < p.pending; ++i) {
            float ms = 0.f;
            cudaEventSynchronize(p.ev[2 * i + 1]);
            if (cudaEventElapsedTime(&ms, p.ev[2 * i], p.ev[2 * i + 1]) == cudaSuccess) {
                p.total_ms += ms;
                p.count++;
            }
        }
        p.pending = 0;
    }
}

template <typename T>
void launch_update(bella_ws *ws, cudaStream_t s) {
    prof_begin(ws, PK_UPDATE, s);
    if (std::is_same<T, dfloat>::value) {
        k_update<dfloat><<<ws->grid_vec, VEC_BLOCK, 0, s>>>(ws->n, ws->xdf, ws->pdf[0], ws->pdf[1], ws->rdf,
                                                          ws->vdf[0], ws->vdf[1], ws->tdf, ws->rhdf,
                                                          ws->ks, ws->partials, ws->counter);
    } else if (std::is_same<T, double>::value) {
        k_update<double><<<ws->grid_vec, VEC_BLOCK, 0, s>>>(ws->n, ws->x64v, ws->p64[0], ws->p64[1], ws->r64k,
                                                          ws->v64[0], ws->v64[1], ws->t64, ws->rh64,
                                                          ws->ks, ws->partials, ws->counter);
    } else {
        k_update<float><<<ws->grid_vec, VEC_BLOCK, 0, s>>>(ws->n, ws->x32, ws->p32[0], ws->p32[1], ws->r32,
                                                         ws->v32[0], ws->v32[1], ws->t32, ws->rh32,
                                                         ws->ks, ws->partials, ws->counter);
    }
    prof_end(ws, PK_UPDATE, s);
    ws->launches++;
}
template void launch_update<float>(bella_ws *, cudaStream_t);
template void launch_update<double>(bella_ws *, cudaStream_t);
template void launch_update<dfloat>(bella_ws *, cudaStream_t);

static __device__ void init_state(KState *ks, double rr, double atol, double rhotol, int maxiter) {
    ks->rho = rr;           // r^ = r  ->  rho = ||r||^2
    ks->rho0 = rr;
    ks->rho_prev = 1.0;
    ks->rr = rr;
    ks->alpha = 1.0;
    ks->omega = 1.0;
    ks->beta = 0.0;
    ks->atol = atol;
    ks->rhotol = rhotol;
    ks->iter = 0;
    ks->maxiter = maxiter;
    ks->early = 0;
    ks->done = 0;
    ks->status = BELLA_MAXITER;
    ks->pad[0] = 0;
    ks->pad[1] = 0;
    if (!isfinite(rr)) { ks->status = BELLA_NONFINITE; ks->done = 1; }
    else if (sqrt(rr) <= atol) { ks->status = BELLA_OK; ks->done = 1; }
    else if (maxiter <= 0) { ks->status = BELLA_MAXITER; ks->done = 1; }
    else if (!(rr > 0.0)) { ks->status = BELLA_BREAKDOWN; ks->done = 1; }
}

// FP64 solve start.  x_given = 0: x = 0, r = b.  x_given = 1: r already
// holds b - A x.  r^ = r.  atol = max(atol_user, tol*||b||) and the scipy
// 1.7 legacy exit ||b|| <= tol -> x = 0 (x0 = 0 only).
__global__ void __launch_bounds__(VEC_BLOCK)
k_init64(long long n, const double *b, double *x, double *r, double *rh, int x_given, double tol,
         double atol_user, int maxiter, KState *ks, double *partials, unsigned *counter) {
    DD a0, a1;
    a0.zero(); a1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const double bg = b[g];
        double rg;
        if (!x_given) { x[g] = 0.0; rg = bg; r[g] = rg; }
        else rg = r[g];
        rh[g] = rg;
        a0.add_prod(rg, rg);
        a1.add_prod(bg, bg);
    }
    double vv[2] = {a0.value(), a1.value()}, tot[2];
    if (!grid_sum<2>(vv, partials, counter, tot)) return;
    if (threadIdx.x != 0) return;
    const double bnorm = sqrt(tot[1]);
    double atol = tol * bnorm;
    if (atol_user > atol) atol = atol_user;
    init_state(ks, tot[0], atol, 4.930380657631324e-32 /* eps64^2 */, maxiter);
    ks->dot_aux = bnorm;
    if (bnorm == 0.0 || (!x_given && bnorm <= tol)) { ks->status = BELLA_OK; ks->done = 1; }
}

// Double-float solve start.  x_given = 0: x = 0, r = b.  x_given = 1: r64 holds
// b - A x (FP64) and x is the FP64 start.  r^ = r.  Same thresholds as k_init64.
__global__ void __launch_bounds__(VEC_BLOCK)
k_init_df(long long n, const double *b, const double *x64, const double *r64, dfloat *x, dfloat *r,
          dfloat *rh, int x_given, double tol, double atol_user, int maxiter, KState *ks, double *partials,
          unsigned *counter) {
    DD a0, a1;
    a0.zero(); a1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const double bg = b[g];
        const double rg = x_given ? r64[g] : bg;
        const dfloat rd(rg);
        r[g] = rd;
        rh[g] = rd;
        x[g] = x_given ? dfloat(x64[g]) : dfloat(0.f, 0.f);
        a0.add_prod(rg, rg);
        a1.add_prod(bg, bg);
    }
    double vv[2] = {a0.value(), a1.value()}, tot[2];
    if (!grid_sum<2>(vv, partials, counter, tot)) return;
    if (threadIdx.x != 0) return;
    const double bnorm = sqrt(tot[1]);
    double atol = tol * bnorm;
    if (atol_user > atol) atol = atol_user;
    init_state(ks, tot[0], atol, 4.930380657631324e-32, maxiter);
    ks->dot_aux = bnorm;
    if (bnorm == 0.0 || (!x_given && bnorm <= tol)) { ks->status = BELLA_OK; ks->done = 1; }
}

// Residual replacement (reliable update): r = b - A x computed in FP64
// replaces the recursive double-float residual and the iteration continues
// with the same r^ and p; rho and beta are recomputed from the new r.  After
// an early (||s||) exit the omega step is missing, so the caller restarts.
__global__ void __launch_bounds__(VEC_BLOCK)
k_replace_df(long long n, const double *r64, dfloat *r, const dfloat *rh, KState *ks, double *partials,
             unsigned *counter) {
    DFAcc a0, a1;
    a0.zero(); a1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const dfloat rd(r64[g]);
        r[g] = rd;
        a0.add_prod(rh[g], rd);
        a1.add_prod(rd, rd);
    }
    double vv[2] = {a0.value(), a1.value()}, tot[2];
    if (!grid_sum<2>(vv, partials, counter, tot)) return;
    if (threadIdx.x != 0) return;
    ks->rr = tot[1];
    ks->done = 0;
    ks->status = BELLA_MAXITER;
    ks->pad[0] = 0;
    if (ks->early || ks->omega == 0.0 || !isfinite(tot[0])) { ks->pad[1] = 1; ks->done = 1; return; }
    ks->rho = tot[0];
    ks->beta = (ks->rho / ks->rho_prev) * (ks->alpha / ks->omega);
    if (sqrt(tot[1]) <= ks->atol) { ks->status = BELLA_OK; ks->done = 1; }
    else if (ks->iter >= ks->maxiter) { ks->status = BELLA_MAXITER; ks->done = 1; }
}

// x (FP64 output) = double-float solution
__global__ void k_df_to_f64(long long n, const dfloat *xd, double *x) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x)
        x[g] = xd[g].to_double();
}

// FP32 inner solve start (iterative refinement): r32 = r64 / scale, r^ = r32, x32 = 0.
__global__ void __launch_bounds__(VEC_BLOCK)
k_init32(long long n, const double *r64, double inv_scale, float *r, float *rh, float *x,
         double atol, int maxiter, KState *ks, double *partials, unsigned *counter) {
    DF a0;
    a0.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x) {
        const float rg = (float)(r64[g] * inv_scale);
        r[g] = rg;
        rh[g] = rg;
        x[g] = 0.f;
        a0.add_prod(rg, rg);
    }
    double vv[1] = {a0.value()}, tot[1];
    if (!grid_sum<1>(vv, partials, counter, tot)) return;
    if (threadIdx.x == 0) init_state(ks, tot[0], atol, 4.930380657631324e-32, maxiter);
}

// The null modes are sign patterns of a node's index parities p (bit 0: i, 1: j,
// 2: k), so every sum over nodes weighted by a mode is a signed combination of the
// 8 parity-class sums, and every shift by a combination of modes is one constant
// per class: one FP64 operation per node instead of one per mode (GB300's FP64
// pipe bounds these passes).  The class sums live in shared memory, one slot per
// class and thread.

// x64 += scale * x32, and <z e_k, x64> for every null mode (projection)
__global__ void __launch_bounds__(VEC_BLOCK)
k_ir_update(long long n, double *x64, const float *x32, double scale, const double *z, NullSpace ns,
            KState *ks, double *partials, unsigned *counter) {
    __shared__ double cls[8][VEC_BLOCK];
    const int tid = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 8; ++q) cls[q][tid] = 0.0;
    for (long long g = blockIdx.x * (long long)blockDim.x + tid; g < n; g += (long long)gridDim.x * blockDim.x) {
        const double xn = x64[g] + scale * (double)x32[g];
        x64[g] = xn;
        if (ns.nm) cls[node_parity(ns, g)][tid] += z[g] * xn;
    }
    if (!ns.nm) return;
    double acc[MAXNULL];
#pragma unroll
    for (int m = 0; m < MAXNULL; ++m) {
        acc[m] = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (m < ns.nm) acc[m] += null_mode_p(ns, m, q) * cls[q][tid];
    }
    double tot[MAXNULL];
    if (!grid_sum<MAXNULL>(acc, partials, counter, tot)) return;
    if (tid == 0) {
        for (int k = 0; k < ns.nm; ++k) {
            ks->nd[k] = tot[k];
            double c = 0.0;
            for (int l = 0; l < ns.nm; ++l) c += ns.ginv[k * MAXNULL + l] * tot[l];
            ks->cnull[k] = c;
        }
    }
}

// x64 -= sum_l c_l e_l: removes the null-space component, keeping x in the
// operator's range where the exact Krylov solution from x0 = 0 lies
__global__ void k_null_shift(long long n, double *x64, const KState *ks, NullSpace ns) {
    __shared__ double D[8];                       // the shift of each parity class
    if (threadIdx.x < 8) {
        double d = 0.0;
        for (int m = 0; m < ns.nm; ++m) d += ks->cnull[m] * null_mode_p(ns, m, threadIdx.x);
        D[threadIdx.x] = d;
    }
    __syncthreads();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x)
        x64[g] -= D[node_parity(ns, g)];
}

// the 8 parity-class sums of z -> ks->nd[0..7]; the Gram matrix of the modes
// follows from them, G_kl = sum_p e_k(p) e_l(p) Z_p
__global__ void __launch_bounds__(VEC_BLOCK)
k_null_classes(long long n, const double *z, NullSpace ns, KState *ks, double *partials, unsigned *counter) {
    __shared__ double cls[8][VEC_BLOCK];
    const int tid = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 8; ++q) cls[q][tid] = 0.0;
    for (long long g = blockIdx.x * (long long)blockDim.x + tid; g < n; g += (long long)gridDim.x * blockDim.x)
        cls[node_parity(ns, g)][tid] += z[g];
    double a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = cls[q][tid];
    double tot[8];
    if (!grid_sum<8>(a, partials, counter, tot)) return;
    if (tid == 0)
        for (int q = 0; q < 8; ++q) ks->nd[q] = tot[q];
}

// generic FP64 dot -> ks->dot_aux
__global__ void __launch_bounds__(VEC_BLOCK)
k_dot64(long long n, const double *a, const double *b, KState *ks, double *partials, unsigned *counter) {
    DD a0;
    a0.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
         g += (long long)gridDim.x * blockDim.x)
        a0.add_prod(a[g], b ? b[g] : 1.0);
    double vv[1] = {a0.value()}, tot[1];
    if (!grid_sum<1>(vv, partials, counter, tot)) return;
    if (threadIdx.x == 0) ks->dot_aux = tot[0];
}

}  // namespace bella

// ============================================================================
// C ABI
// ============================================================================
using namespace bella;

extern "C" {

const char *bella_last_error(void) { return g_err.c_str(); }

const char *bella_status_string(int st) {
    switch (st) {
        case BELLA_OK: return "converged";
        case BELLA_MAXITER: return "iteration limit reached";
        case BELLA_BREAKDOWN: return "breakdown (rho or omega below limit)";
        case BELLA_NONFINITE: return "non-finite residual";
        case BELLA_TIMEOUT: return "timeout";
        case BELLA_EINVAL: return "invalid argument";
        case BELLA_ECUDA: return "CUDA error";
        case BELLA_ENOOP: return "no operator set";
        default: return "unknown status";
    }
}

int bella_version(void) { return 100; }

long long bella_ws_launches(const bella_ws *ws) { return ws ? ws->launches : 0; }

int bella_ws_create(bella_ws **out, int device) {
    if (!out) return set_err(BELLA_EINVAL, "bella_ws_create: null output pointer");
    *out = nullptr;
    BELLA_CUDA(cudaSetDevice(device));
    bella_ws *ws = (bella_ws *)calloc(1, sizeof(bella_ws));
    if (!ws) return set_err(BELLA_EINVAL, "bella_ws_create: out of host memory");
    ws->device = device;
    int rc = cuda_check(cudaMalloc(&ws->ks, sizeof(KState)), "cudaMalloc(ks)");
    if (rc == BELLA_OK) rc = cuda_check(cudaMallocHost(&ws->ks_host, sizeof(KState)), "cudaMallocHost(ks)");
    if (rc == BELLA_OK) rc = cuda_check(cudaMalloc(&ws->counter, 64), "cudaMalloc(counter)");
    if (rc == BELLA_OK) rc = cuda_check(cudaMemset(ws->counter, 0, 64), "cudaMemset(counter)");
    if (rc == BELLA_OK)
        rc = cuda_check(cudaMalloc(&ws->partials, sizeof(double) * NQ * MAXGRID), "cudaMalloc(partials)");
    if (rc == BELLA_OK) rc = cuda_check(cudaMemset(ws->ks, 0, sizeof(KState)), "cudaMemset(ks)");
    if (rc != BELLA_OK) {
        bella_ws_destroy(ws);
        return rc;
    }
    *out = ws;
    return BELLA_OK;
}

static void free_op(bella_ws *ws) {
    cudaFree(ws->a64); cudaFree(ws->a32);
    cudaFree(ws->dinv64); cudaFree(ws->hc64); cudaFree(ws->z64);
    cudaFree(ws->dinv32); cudaFree(ws->hc32);
    cudaFree(ws->adf); cudaFree(ws->dinvdf); cudaFree(ws->hcdf);
    ws->a64 = nullptr; ws->a32 = nullptr; ws->dinv64 = ws->hc64 = ws->z64 = nullptr;
    ws->dinv32 = ws->hc32 = nullptr;
    ws->adf = ws->dinvdf = ws->hcdf = nullptr;
}

int bella_ws_destroy(bella_ws *ws) {
    if (!ws) return BELLA_OK;
    cudaSetDevice(ws->device);
    if (ws->prof) bella_ws_profile(ws, 0);
    bella_spectral3d_destroy(ws->sp_cache);
    free_op(ws);
    cudaFree(ws->proj_buf);
    cudaFree(ws->fg_v);
    cudaFree(ws->fg_z);
    cudaFree(ws->fg_part);
    cudaFree(ws->fg_dev);
    cudaFree(ws->vbase);
    cudaFree(ws->partials);
    cudaFree(ws->counter);
    cudaFree(ws->ks);
    if (ws->ks_host) cudaFreeHost(ws->ks_host);
    free(ws);
    return BELLA_OK;
}

// carve the Krylov vectors for n unknowns out of one allocation
static int ensure_vectors(bella_ws *ws, long long n) {
    if (ws->cap >= n && ws->vbase) return BELLA_OK;
    cudaFree(ws->vbase);
    ws->vbase = nullptr;
    const long long np = (n + 63) / 64 * 64;   // 256-byte aligned slices
    const size_t bytes = (size_t)np * (8 * 9 + 4 * 11 + 8 * 8);
    BELLA_CUDA(cudaMalloc(&ws->vbase, bytes));
    char *p = (char *)ws->vbase;
    auto take64 = [&](double **d) { *d = (double *)p; p += np * 8; };
    auto take32 = [&](float **f) { *f = (float *)p; p += np * 4; };
    take64(&ws->r64); take64(&ws->x64v); take64(&ws->r64k); take64(&ws->rh64);
    take64(&ws->p64[0]); take64(&ws->p64[1]); take64(&ws->v64[0]); take64(&ws->v64[1]); take64(&ws->t64);
    take32(&ws->r32); take32(&ws->rh32); take32(&ws->p32[0]); take32(&ws->p32[1]);
    take32(&ws->v32[0]); take32(&ws->v32[1]); take32(&ws->t32); take32(&ws->x32);
    take32(&ws->s32); take32(&ws->ph32); take32(&ws->sh32);
    auto takedf = [&](dfloat **d) { *d = (dfloat *)p; p += np * 8; };
    takedf(&ws->rdf); takedf(&ws->rhdf); takedf(&ws->pdf[0]); takedf(&ws->pdf[1]);
    takedf(&ws->vdf[0]); takedf(&ws->vdf[1]); takedf(&ws->tdf); takedf(&ws->xdf);
    ws->cap = n;
    return BELLA_OK;
}

// Null modes of a singular (pseudo-incompressible) operator and the inverse of
// their Gram matrix.  A checkerboard on a periodic axis needs an even period.
static int setup_null_space(bella_ws *ws, cudaStream_t s, int xper, int yper, int zper) {
    NullSpace &ns = ws->ns;
    memset(&ns, 0, sizeof(ns));
    ns.ndim = ws->ndim;
    ns.nx = ws->nx; ns.ny = ws->ny; ns.nz = ws->nz > 0 ? ws->nz : 1;
    if (!ws->singular) return BELLA_OK;
    const int nn[3] = {ws->nx, ws->ny, ws->nz};
    const int per[3] = {xper, yper, zper};
    auto ok = [&](int axis) { return !per[axis] || ((nn[axis] - 1) % 2 == 0); };
    auto add = [&](int a, int b, int c) {
        ns.sx[ns.nm] = (signed char)a; ns.sy[ns.nm] = (signed char)b; ns.sz[ns.nm] = (signed char)c; ns.nm++;
    };
    add(1, 1, 1);
    if (ws->ndim == 2) {
        if (ok(0) && ok(1)) add(-1, -1, 1);
    } else {
        if (ok(0) && ok(1)) add(-1, -1, 1);
        if (ok(0) && ok(2)) add(-1, 1, -1);
        if (ok(1) && ok(2)) add(1, -1, -1);
        if (ok(0) && ok(1) && ok(2)) add(-1, -1, -1);
    }
    const int nm = ns.nm;
    double G[MAXNULL * MAXNULL];
    k_null_classes<<<ws->grid_vec, VEC_BLOCK, 0, s>>>(ws->n, ws->z64, ns, ws->ks, ws->partials, ws->counter);
    ws->launches++;
    BELLA_CUDA(cudaGetLastError());
    BELLA_CUDA(cudaMemcpyAsync(ws->ks_host, ws->ks, sizeof(KState), cudaMemcpyDeviceToHost, s));
    BELLA_CUDA(cudaStreamSynchronize(s));
    auto sign = [&](int m, int p) {                   // null_mode_p on the host
        int par = 0;
        if (ns.sx[m] < 0) par ^= p & 1;
        if (ns.sy[m] < 0) par ^= (p >> 1) & 1;
        if (ns.sz[m] < 0) par ^= (p >> 2) & 1;
        return par ? -1.0 : 1.0;
    };
    for (int k = 0; k < nm; ++k)
        for (int l = 0; l < nm; ++l) {
            double g = 0.0;
            for (int q = 0; q < 8; ++q) g += sign(k, q) * sign(l, q) * ws->ks_host->nd[q];
            G[k * nm + l] = g;
        }
    // Gauss-Jordan inverse with partial pivoting (nm <= 8)
    double A[MAXNULL][2 * MAXNULL];
    for (int r = 0; r < nm; ++r)
        for (int c = 0; c < 2 * nm; ++c) A[r][c] = c < nm ? G[r * nm + c] : (c - nm == r ? 1.0 : 0.0);
    for (int c = 0; c < nm; ++c) {
        int piv = c;
        for (int r = c + 1; r < nm; ++r) if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
        if (A[piv][c] == 0.0) return set_err(BELLA_EINVAL, "null-space Gram matrix is singular");
        if (piv != c) for (int q = 0; q < 2 * nm; ++q) { double t = A[c][q]; A[c][q] = A[piv][q]; A[piv][q] = t; }
        const double d = A[c][c];
        for (int q = 0; q < 2 * nm; ++q) A[c][q] /= d;
        for (int r = 0; r < nm; ++r) {
            if (r == c) continue;
            const double f = A[r][c];
            if (f != 0.0) for (int q = 0; q < 2 * nm; ++q) A[r][q] -= f * A[c][q];
        }
    }
    for (int r = 0; r < nm; ++r)
        for (int c = 0; c < nm; ++c) ns.ginv[r * MAXNULL + c] = A[r][nm + c];
    return BELLA_OK;
}

int bella_op2d_set(bella_ws *ws, const bella_op2d *op, void *stream) {
    if (!ws || !op) return set_err(BELLA_EINVAL, "bella_op2d_set: null argument");
    if (op->nx < 3 || op->ny < 3) return set_err(BELLA_EINVAL, "bella_op2d_set: nx, ny must be >= 3");
    if (!op->hplusx || !op->hplusy || !op->cxx || !op->cyy || !op->diag_inv)
        return set_err(BELLA_EINVAL, "bella_op2d_set: hplusx, hplusy, cxx, cyy, diag_inv are required");
    if (!(op->dx > 0.0) || !(op->dy > 0.0)) return set_err(BELLA_EINVAL, "bella_op2d_set: dx, dy must be > 0");
    if ((long long)(op->nx + 1) * (op->ny + 1) >= (1LL << 31))   // node indices are 32-bit in the null space
        return set_err(BELLA_EINVAL, "bella_op2d_set: (nx+1)(ny+1) must be below 2^31");
    if (op->x_wall < 0 || op->x_wall > 1 || op->y_wall < 0 || op->y_wall > BELLA_Y_MIRROR)
        return set_err(BELLA_EINVAL, "bella_op2d_set: x_wall must be 0 or 1, y_wall 0, 1 or BELLA_Y_MIRROR");
    if (op->y_wall == BELLA_Y_MIRROR && op->x_wall)
        return set_err(BELLA_EINVAL, "bella_op2d_set: the mirrored y boundary (LAMB_BDRY) has a periodic x axis");
    BELLA_CUDA(cudaSetDevice(ws->device));
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)op->nx * op->ny;
    const size_t ncell = (size_t)(op->nx + 1) * (op->ny + 1);
    if (ws->ndim != 2 || ws->nx != op->nx || ws->ny != op->ny) {
        free_op(ws);
        BELLA_CUDA(cudaMalloc(&ws->a64, 4 * ncell * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->a32, 4 * ncell * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->dinv64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->hc64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->z64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->dinv32, n * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->hc32, n * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->adf, 4 * ncell * sizeof(dfloat)));
        BELLA_CUDA(cudaMalloc(&ws->dinvdf, n * sizeof(dfloat)));
        BELLA_CUDA(cudaMalloc(&ws->hcdf, n * sizeof(dfloat)));
    }
    int rc = ensure_vectors(ws, n);
    if (rc != BELLA_OK) return rc;
    ws->ndim = 2;
    ws->nz = 1;
    ws->nx = op->nx;
    ws->ny = op->ny;
    ws->n = n;
    ws->cross = (op->cxy != nullptr || op->cyx != nullptr) ? 1 : 0;
    ws->has_hc = op->hcenter != nullptr ? 1 : 0;
    ws->ymirror = op->y_wall == BELLA_Y_MIRROR ? 1 : 0;
    // the null space projection is that of the wrapped/walled operator: not applied with the mirror
    ws->singular = (!ws->has_hc && !ws->cross && !ws->ymirror) ? 1 : 0;
    ws->per[0] = op->x_wall ? 0 : 1; ws->per[1] = op->y_wall ? 0 : 1; ws->per[2] = 0;
    ws->grid_stencil = stencil_grid(op->nx, op->ny);
    ws->grid_vec = vec_grid(n);
    rc = op2d_pack(ws, op, s);
    if (rc != BELLA_OK) return cuda_check(cudaGetLastError(), "op2d_pack");
    rc = setup_null_space(ws, s, op->x_wall ? 0 : 1, op->y_wall == 0 ? 1 : 0, 0);
    if (rc != BELLA_OK) return rc;
    return BELLA_OK;
}

int bella_op3d_set(bella_ws *ws, const bella_op3d *op, void *stream) {
    if (!ws || !op) return set_err(BELLA_EINVAL, "bella_op3d_set: null argument");
    if (op->nx < 3 || op->ny < 3 || op->nz < 3) return set_err(BELLA_EINVAL, "bella_op3d_set: nx, ny, nz must be >= 3");
    if (!op->hplusx || !op->hplusy || !op->hplusz || !op->diag_inv)
        return set_err(BELLA_EINVAL, "bella_op3d_set: hplusx, hplusy, hplusz, diag_inv are required");
    if (!(op->dx > 0.0) || !(op->dy > 0.0) || !(op->dz > 0.0))
        return set_err(BELLA_EINVAL, "bella_op3d_set: dx, dy, dz must be > 0");
    const size_t ncell = (size_t)(op->nx + 1) * (op->ny + 1) * (op->nz + 1);
    if (ncell >= (size_t)1 << 31)   // the stencil indexes nodes and cells with 32-bit offsets
        return set_err(BELLA_EINVAL, "bella_op3d_set: (nx+1)(ny+1)(nz+1) must be below 2^31");
    BELLA_CUDA(cudaSetDevice(ws->device));
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)op->nx * op->ny * op->nz;
    if (ws->ndim != 3 || ws->nx != op->nx || ws->ny != op->ny || ws->nz != op->nz) {
        free_op(ws);
        BELLA_CUDA(cudaMalloc(&ws->a64, 5 * ncell * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->a32, 5 * ncell * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->adf, 5 * ncell * sizeof(dfloat)));
        BELLA_CUDA(cudaMalloc(&ws->dinv64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->hc64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->z64, n * sizeof(double)));
        BELLA_CUDA(cudaMalloc(&ws->dinv32, n * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->hc32, n * sizeof(float)));
        BELLA_CUDA(cudaMalloc(&ws->dinvdf, n * sizeof(dfloat)));
        BELLA_CUDA(cudaMalloc(&ws->hcdf, n * sizeof(dfloat)));
    }
    int rc = ensure_vectors(ws, n);
    if (rc != BELLA_OK) return rc;
    ws->ndim = 3;
    ws->nx = op->nx; ws->ny = op->ny; ws->nz = op->nz;
    ws->n = n;
    ws->cross = op->corrf != 0.0 ? 1 : 0;
    ws->has_hc = op->hcenter != nullptr ? 1 : 0;
    ws->ymirror = 0;
    ws->singular = (!ws->has_hc && !ws->cross) ? 1 : 0;
    ws->per[0] = op->x_wall ? 0 : 1; ws->per[1] = op->y_wall ? 0 : 1; ws->per[2] = op->z_wall ? 0 : 1;
    ws->grid_stencil = stencil3d_grid(op->nx, op->ny, op->nz);
    ws->grid_vec = vec_grid(n);
    rc = op3d_pack(ws, op, s);
    if (rc != BELLA_OK) return cuda_check(cudaGetLastError(), "op3d_pack");
    return setup_null_space(ws, s, op->x_wall ? 0 : 1, op->y_wall ? 0 : 1, op->z_wall ? 0 : 1);
}

int bella_apply_f64(bella_ws *ws, const double *x, double *y, void *stream) {
    if (!ws || !x || !y) return set_err(BELLA_EINVAL, "bella_apply_f64: null argument");
    if (ws->ndim == 0) return set_err(BELLA_ENOOP, "bella_apply_f64: no operator set");
    op_apply(ws, 0, x, y, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "bella_apply_f64");
}

int bella_apply_f32(bella_ws *ws, const float *x, float *y, void *stream) {
    if (!ws || !x || !y) return set_err(BELLA_EINVAL, "bella_apply_f32: null argument");
    if (ws->ndim == 0) return set_err(BELLA_ENOOP, "bella_apply_f32: no operator set");
    op_apply(ws, 1, x, y, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "bella_apply_f32");
}

void bella_solve_opts_default(bella_solve_opts *o) {
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->tol = 1e-8;
    o->atol = 0.0;
    o->maxiter = 6000;
    o->precision = 1;
    o->x0_zero = 1;
    o->project_null = 1;
    o->inner_tol = 1e-5;
    o->max_outer = 30;
    o->check_every = 16;
    o->timeout_s = 0.0;
}

static int sync_state(bella_ws *ws, cudaStream_t s) {
    BELLA_CUDA(cudaMemcpyAsync(ws->ks_host, ws->ks, sizeof(KState), cudaMemcpyDeviceToHost, s));
    BELLA_CUDA(cudaStreamSynchronize(s));
    prof_harvest(ws);
    return BELLA_OK;
}

int bella_ws_profile(bella_ws *ws, int enable) {
    if (!ws) return set_err(BELLA_EINVAL, "bella_ws_profile: null workspace");
    BELLA_CUDA(cudaSetDevice(ws->device));
    if (enable && !ws->prof) {
        for (int k = 0; k < 4; ++k)
            for (int i = 0; i < 2 * 256; ++i) BELLA_CUDA(cudaEventCreate(&ws->profk[k].ev[i]));
    }
    if (!enable && ws->prof) {
        prof_harvest(ws);
        for (int k = 0; k < 4; ++k)
            for (int i = 0; i < 2 * 256; ++i) cudaEventDestroy(ws->profk[k].ev[i]);
    }
    ws->prof = enable ? 1 : 0;
    for (int k = 0; k < 4; ++k) { ws->profk[k].pending = 0; ws->profk[k].total_ms = 0.0; ws->profk[k].count = 0; }
    return BELLA_OK;
}

int bella_ws_kernel_time(bella_ws *ws, int kind, double *total_ms, long long *count) {
    if (!ws || kind < 0 || kind > 3 || !total_ms || !count)
        return set_err(BELLA_EINVAL, "bella_ws_kernel_time: bad argument");
    prof_harvest(ws);
    *total_ms = ws->profk[kind].total_ms;
    *count = ws->profk[kind].count;
    return BELLA_OK;
}

// run BiCGStab iterations (precision prec) until the device state is done
static int run_inner(bella_ws *ws, int prec, const bella_solve_opts *o, cudaStream_t s,
                     std::chrono::steady_clock::time_point t0, int *timed_out) {
    const int blk = o->check_every > 0 ? o->check_every : 16;
    *timed_out = 0;
    for (;;) {
        int rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        if (ws->ks_host->done) return BELLA_OK;
        if (o->timeout_s > 0.0) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > o->timeout_s) { *timed_out = 1; return BELLA_OK; }
        }
        for (int k = 0; k < blk; ++k) op_iteration(ws, prec, s);
        BELLA_CUDA(cudaGetLastError());
    }
}

// Double-float iterations with a divergence guard: at every host check the
// iterate with the smallest recursive residual so far is kept in FP64 (xbest,
// refreshed when the residual has halved), and the run stops with *diverged
// set when the recursive residual norm is non-finite or has grown a
// million-fold above that best value.
static int run_inner_guarded(bella_ws *ws, const bella_solve_opts *o, cudaStream_t s,
                             std::chrono::steady_clock::time_point t0, int *timed_out, int *diverged, double *xbest,
                             double *best_rr) {
    const int blk = o->check_every > 0 ? o->check_every : 16;
    *timed_out = 0;
    *diverged = 0;
    for (;;) {
        int rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        const double rr = ws->ks_host->rr;
        if (!isfinite(rr) || (isfinite(*best_rr) && rr > 1e12 * *best_rr)) {
            *diverged = 1;
            return BELLA_OK;
        }
        if (rr < 0.25 * *best_rr) {
            k_df_to_f64<<<ws->grid_vec, VEC_BLOCK, 0, s>>>(ws->n, ws->xdf, xbest);
            ws->launches++;
            *best_rr = rr;
        }
        if (ws->ks_host->done) return BELLA_OK;
        if (o->timeout_s > 0.0) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > o->timeout_s) { *timed_out = 1; return BELLA_OK; }
        }
        for (int k = 0; k < blk; ++k) op_iteration(ws, 2, s);
        BELLA_CUDA(cudaGetLastError());
    }
}

// FP64 BiCGStab with scipy's control flow; x is the solution in place.
// x_given = 0 starts from x = 0.  Fills iterations/status/bnorm/matvecs.
static int solve_fp64(bella_ws *ws, const double *b, double *x, const bella_solve_opts &o, int x_given,
                      int maxiter, bella_solve_stats *st, cudaStream_t s,
                      std::chrono::steady_clock::time_point t0) {
    const long long n = ws->n;
    int timed_out = 0;
    if (x_given) op_resid(ws, 0, x, b, ws->r64k, s);
    k_init64<<<ws->grid_vec, VEC_BLOCK, 0, s>>>(n, b, x, ws->r64k, ws->rh64, x_given, o.tol, o.atol, maxiter,
                                                ws->ks, ws->partials, ws->counter);
    ws->launches++;
    BELLA_CUDA(cudaGetLastError());
    double *saved = ws->x64v;            // the update kernel writes ws->x64v
    ws->x64v = x;
    int rc = run_inner(ws, 0, &o, s, t0, &timed_out);
    ws->x64v = saved;
    if (rc != BELLA_OK) return rc;
    st->iterations += ws->ks_host->iter;
    st->status = timed_out ? BELLA_TIMEOUT : ws->ks_host->status;
    st->bnorm = ws->ks_host->dot_aux;
    st->matvecs += 2 * ws->ks_host->iter + (x_given ? 1 : 0);
    st->detail = ws->ks_host->pad[0];
    return BELLA_OK;
}

// Double-float BiCGStab (scipy control flow) on the FP32 pipe; x in/out FP64.
// Convergence is only accepted on the FP64 true residual: when the recursive
// double-float residual meets the tolerance, b - A x is recomputed in FP64 and,
// if it is still too large, replaces the recursive one (reliable update) and
// the iteration goes on (restarting after an early ||s|| exit).
static int solve_df(bella_ws *ws, const double *b, double *x, const bella_solve_opts &o, int x_given,
                    int maxiter, bella_solve_stats *st, cudaStream_t s,
                    std::chrono::steady_clock::time_point t0) {
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    int timed_out = 0;
    if (x_given) op_resid(ws, 0, x, b, ws->r64, s);
    k_init_df<<<gv, VEC_BLOCK, 0, s>>>(n, b, x, ws->r64, ws->xdf, ws->rdf, ws->rhdf, x_given, o.tol, o.atol,
                                       maxiter, ws->ks, ws->partials, ws->counter);
    ws->launches++;
    BELLA_CUDA(cudaGetLastError());
    int rc, replaced = 0, restarts = 0, iters_before = 0, rescues = 0;
    bool true_too_large = false, gave_up = false;
    st->matvecs += x_given ? 1 : 0;
    double best_rr = INFINITY;
    for (;;) {
        int diverged = 0;
        rc = run_inner_guarded(ws, &o, s, t0, &timed_out, &diverged, ws->x64v, &best_rr);
        if (rc != BELLA_OK) return rc;
        const KState k = *ws->ks_host;
        st->detail = k.pad[0];
        if (diverged || (k.status == BELLA_NONFINITE && isfinite(best_rr))) {
            // the recursion blew up: continue from the best iterate seen, with a
            // fresh Krylov process, a few times; then return that iterate
            const double bnorm = k.dot_aux;
            BELLA_CUDA(cudaMemcpyAsync(x, ws->x64v, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            iters_before += k.iter;
            const int left = maxiter - iters_before;
            if (rescues >= 4 || left <= 0 || timed_out) { gave_up = true; break; }
            rescues++;
            op_resid(ws, 0, x, b, ws->r64, s);
            st->matvecs += 1;
            k_init_df<<<gv, VEC_BLOCK, 0, s>>>(n, b, x, ws->r64, ws->xdf, ws->rdf, ws->rhdf, 1, o.tol, o.atol, left,
                                               ws->ks, ws->partials, ws->counter);
            ws->launches++;
            rc = sync_state(ws, s);
            if (rc != BELLA_OK) return rc;
            ws->ks_host->dot_aux = bnorm;
            best_rr = INFINITY;
            continue;
        }
        k_df_to_f64<<<gv, VEC_BLOCK, 0, s>>>(n, ws->xdf, x);
        ws->launches++;
        if (timed_out || k.status != BELLA_OK || k.iter >= maxiter) break;
        const double bnorm = k.dot_aux, atol = k.atol;
        op_resid(ws, 0, x, b, ws->r64, s);
        st->matvecs += 1;
        rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        const double rn = sqrt(ws->ks_host->dot_aux2);
        ws->ks_host->dot_aux = bnorm;
        if (rn <= atol) break;
        if (replaced >= 16) { true_too_large = true; break; }
        replaced++;
        k_replace_df<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r64, ws->rdf, ws->rhdf, ws->ks, ws->partials, ws->counter);
        ws->launches++;
        rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        if (ws->ks_host->pad[1]) {   // early exit: restart the Krylov process from x
            restarts++;
            iters_before += ws->ks_host->iter;
            const int left = maxiter - iters_before;
            if (left <= 0) break;
            k_init_df<<<gv, VEC_BLOCK, 0, s>>>(n, b, x, ws->r64, ws->xdf, ws->rdf, ws->rhdf, 1, o.tol, o.atol, left,
                                               ws->ks, ws->partials, ws->counter);
            ws->launches++;
            rc = sync_state(ws, s);
            if (rc != BELLA_OK) return rc;
            ws->ks_host->dot_aux = bnorm;
        }
    }
    const KState k = *ws->ks_host;
    if (gave_up) {
        st->iterations += iters_before;
        st->status = timed_out ? BELLA_TIMEOUT : BELLA_BREAKDOWN;
        st->detail = 5;                 // the recursion diverged; x is the best iterate seen
        st->bnorm = k.dot_aux;
        st->matvecs += 2 * iters_before;
        st->outer = replaced + rescues;
        return BELLA_OK;
    }
    st->iterations += iters_before + k.iter;
    st->status = timed_out ? BELLA_TIMEOUT : k.status;
    if (st->status == BELLA_OK && true_too_large) st->status = BELLA_MAXITER;   // never on the recursive residual alone
    st->bnorm = k.dot_aux;
    st->matvecs += 2 * (iters_before + k.iter);
    st->outer = replaced + rescues;
    return BELLA_OK;
}

int bella_bicgstab(bella_ws *ws, const double *b, double *x, const bella_solve_opts *opts,
                   bella_solve_stats *stats, void *stream) {
    if (!ws || !b || !x) return set_err(BELLA_EINVAL, "bella_bicgstab: null argument");
    if (ws->ndim == 0) return set_err(BELLA_ENOOP, "bella_bicgstab: no operator set");
    bella_solve_opts o;
    if (opts) o = *opts; else bella_solve_opts_default(&o);
    if (!(o.tol >= 0.0) || o.maxiter < 0) return set_err(BELLA_EINVAL, "bella_bicgstab: bad tol/maxiter");
    BELLA_CUDA(cudaSetDevice(ws->device));
    cudaStream_t s = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    bella_solve_stats st;
    memset(&st, 0, sizeof(st));
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    int rc, timed_out = 0;
    double rn_known = -1.0;                           // >= 0: ||b - A x|| of the returned x, measured

    if (o.precision == 0) {
        rc = solve_fp64(ws, b, x, o, o.x0_zero ? 0 : 1, o.maxiter, &st, s, t0);
        if (rc != BELLA_OK) return rc;
    } else if (o.precision == 2) {
        rc = solve_df(ws, b, x, o, o.x0_zero ? 0 : 1, o.maxiter, &st, s, t0);
        if (rc != BELLA_OK) return rc;
    } else {
        // ---- FP32 BiCGStab inner solves in FP64 iterative refinement ----
        k_dot64<<<gv, VEC_BLOCK, 0, s>>>(n, b, b, ws->ks, ws->partials, ws->counter);
        ws->launches++;
        rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        const double bnorm = sqrt(ws->ks_host->dot_aux);
        st.bnorm = bnorm;
        double target = o.tol * bnorm;
        if (o.atol > target) target = o.atol;
        if (!isfinite(bnorm)) { st.status = BELLA_NONFINITE; goto done; }
        if (o.x0_zero) {
            BELLA_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
            if (bnorm == 0.0 || bnorm <= o.tol) {   // scipy 1.7 legacy exit
                st.status = BELLA_OK;
                goto done;
            }
        }
        {
            NullSpace ns = ws->ns;
            if (!o.project_null) ns.nm = 0;
            const bool proj = ns.nm > 0;
            double rnorm = bnorm;
            if (o.x0_zero) {                          // r = b - A 0 = b exactly: no stencil
                BELLA_CUDA(cudaMemcpyAsync(ws->r64, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            } else {
                op_resid(ws, 0, x, b, ws->r64, s);
                rc = sync_state(ws, s);
                if (rc != BELLA_OK) return rc;
                rnorm = sqrt(ws->ks_host->dot_aux2);
                st.matvecs = 1;
            }
            st.status = BELLA_MAXITER;
            int total = 0;
            bool failed = false;
            for (int outer = 0;; ++outer) {
                if (!isfinite(rnorm)) { st.status = BELLA_NONFINITE; break; }
                if (rnorm <= target) { st.status = BELLA_OK; break; }
                if (total >= o.maxiter) { st.status = BELLA_MAXITER; break; }
                if (outer >= o.max_outer) { failed = true; break; }
                if (timed_out) { st.status = BELLA_TIMEOUT; break; }
                double rel = o.inner_tol;
                const double need = 0.5 * target / rnorm;
                if (need > rel) rel = need;
                k_init32<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r64, 1.0 / rnorm, ws->r32, ws->rh32, ws->x32, rel,
                                                  o.maxiter - total, ws->ks, ws->partials, ws->counter);
                ws->launches++;
                rc = run_inner(ws, 1, &o, s, t0, &timed_out);
                if (rc != BELLA_OK) return rc;
                const int it = ws->ks_host->iter;
                const int inner_status = ws->ks_host->status;
                st.detail = ws->ks_host->pad[0];
                total += it;
                st.matvecs += 2 * it;
                st.outer = outer + 1;
                // a non-finite inner iterate is never applied
                if (inner_status == BELLA_NONFINITE || it == 0) { failed = true; break; }
                // keep the iterate: a rejected correction is undone by copy, not by
                // subtracting it again (which leaves rounding garbage when it is large)
                BELLA_CUDA(cudaMemcpyAsync(ws->x64v, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                k_ir_update<<<gv, VEC_BLOCK, 0, s>>>(n, x, ws->x32, rnorm, ws->z64, ns, ws->ks,
                                                     ws->partials, ws->counter);
                ws->launches++;
                // keep x in the operator's range (A e_k = 0 exactly), before the
                // residual is measured: the shift's rounding moves the FP64 residual
                // by about eps * cond(A), so the residual tested is the returned x's
                if (proj) {
                    k_null_shift<<<gv, VEC_BLOCK, 0, s>>>(n, x, ws->ks, ns);
                    ws->launches++;
                }
                op_resid(ws, 0, x, b, ws->r64, s);
                st.matvecs += 1;
                rc = sync_state(ws, s);
                if (rc != BELLA_OK) return rc;
                const double rnew = sqrt(ws->ks_host->dot_aux2);
                if (!(rnew < rnorm)) {
                    // no progress: restore the iterate and stop refining
                    BELLA_CUDA(cudaMemcpyAsync(x, ws->x64v, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                    failed = true;
                    break;
                }
                rnorm = rnew;
            }
            st.iterations = total;
            if (failed) {
                // fallback from the FP64 iterate, reported in stats.fallback: double-float
                // BiCGStab, which accepts convergence only on the FP64 true residual
                st.fallback = 1;
                const int left = o.maxiter - total;
                rc = solve_df(ws, b, x, o, 1, left > 0 ? left : 0, &st, s, t0);
                if (rc != BELLA_OK) return rc;
            } else {
                rn_known = rnorm;                     // the loop measured the returned x's residual last
            }
        }
    }
done:
    {
        // true FP64 residual of the returned x
        double rn = rn_known;
        if (!(rn >= 0.0)) {
            op_resid(ws, 0, x, b, ws->r64, s);
            rc = sync_state(ws, s);
            if (rc != BELLA_OK) return rc;
            rn = sqrt(ws->ks_host->dot_aux2);
        }
        st.relres = st.bnorm > 0 ? rn / st.bnorm : rn;
        if (!isfinite(rn)) st.status = BELLA_NONFINITE;
    }
    BELLA_CUDA(cudaGetLastError());
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return st.status;
}

}  // extern "C"

// ============================================================================
// Flexible BiCGStab right-preconditioned by the learned CNN (3D operators).
//
// scipy's bicgstab, which the reference calls without a preconditioner
// (second_projection.py:230), takes one through its M argument and applies it
// to p and s; here M is the CNN (nonlinear in its ReLU modes), so the
// iteration is the flexible variant: p^ = M(p), v = A p^, s = r - alpha v,
// s^ = M(s), t = A s^, x += alpha p^ + omega s^.  The scalar recurrences,
// stop tests and breakdown tests are those of the plain solver (finalize_*).
// Inner iterations keep FP32 vectors and the FP32 operator with FP64
// reductions; FP64 iterative refinement on the true residual wraps them as in
// the mixed plain solve.  The plain double-float BiCGStab is the fallback and
// is reported in stats->fallback.  The CNN sees unit-RMS inputs (its scale is
// read on the device, no host synchronisation).
// ============================================================================
namespace bella {

__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_p(long long n, const float *r, float *p, const float *v, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    const bool first = ks->iter == 0;
    const float beta = (float)ks->beta, omega = (float)ks->omega;
    DF d0;
    d0.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        const float pg = first ? r[g] : fmaf(beta, fmaf(-omega, v[g], p[g]), r[g]);
        p[g] = pg;
        d0.add_prod(pg, pg);
    }
    double a[1] = {d0.value()}, tot[1];
    if (!grid_sum<1>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) ks->dot_aux = tot[0];
}

__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_alpha(long long n, const float *rh, const float *v, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    DF d0;
    d0.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x)
        d0.add_prod(rh[g], v[g]);
    double a[1] = {d0.value()}, tot[1];
    if (!grid_sum<1>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) finalize_pdir(ks, tot[0]);
}

// s = r - alpha v, ||s||^2 -> ks->ss and ks->dot_aux (the CNN's scale)
__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_s(long long n, const float *r, const float *v, float *s, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    const float alpha = (float)ks->alpha;
    DF d0;
    d0.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        const float sg = fmaf(-alpha, v[g], r[g]);
        s[g] = sg;
        d0.add_prod(sg, sg);
    }
    double a[1] = {d0.value()}, tot[1];
    if (!grid_sum<1>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) { ks->ss = tot[0]; ks->dot_aux = tot[0]; }
}

__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_omega(long long n, const float *t, const float *s, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    DF d0, d1;
    d0.zero();
    d1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        const float tg = t[g];
        d0.add_prod(tg, s[g]);
        d1.add_prod(tg, tg);
    }
    double a[2] = {d0.value(), d1.value()}, tot[2];
    if (!grid_sum<2>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) finalize_sdir(ks, tot[0], tot[1], ks->ss);
}

// x += alpha p^ + omega s^, r = s - omega t, <r^, r>, ||r||^2
__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_update(long long n, float *x, const float *ph, const float *sh, float *r, const float *s, const float *t,
              const float *rh, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    const float alpha = (float)ks->alpha, omega = ks->early ? 0.f : (float)ks->omega;
    DF d0, d1;
    d0.zero();
    d1.zero();
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        x[g] = fmaf(omega, sh[g], fmaf(alpha, ph[g], x[g]));
        const float rg = fmaf(-omega, t[g], s[g]);
        r[g] = rg;
        d0.add_prod(rh[g], rg);
        d1.add_prod(rg, rg);
    }
    double a[2] = {d0.value(), d1.value()}, tot[2];
    if (!grid_sum<2>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) finalize_update(ks, tot[0], tot[1]);
}

// tmp = in - Ay (in place over Ay) and ||tmp||^2 -> ks->pss: the input of the
// learned correction of the background solve
__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_corr_in(long long n, const float *in, float *Ay, KState *ks, double *partials, unsigned *counter) {
    if (ks->done) return;
    DF d0;
    d0.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; g0 < n; g0 += 4 * stride) {
        float a[4], b[4];                             // four elements, loads first
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long g = g0 + u * stride;
            a[u] = g < n ? in[g] : 0.f;
            b[u] = g < n ? Ay[g] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long g = g0 + u * stride;
            if (g < n) {
                const float d = a[u] - b[u];
                Ay[g] = d;
                d0.add_prod(d, d);
            }
        }
    }
    double a[1] = {d0.value()}, tot[1];
    if (!grid_sum<1>(a, partials, counter, tot)) return;
    if (threadIdx.x == 0) ks->pss = tot[0];
}

__global__ void __launch_bounds__(VEC_BLOCK)
k_flex_add(long long n, float *out, const float *add, const KState *ks) {
    if (ks->done) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; g0 < n; g0 += 4 * stride) {
        float a[4], b[4];                             // four elements, loads first
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long g = g0 + u * stride;
            a[u] = g < n ? out[g] : 0.f;
            b[u] = g < n ? add[g] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long g = g0 + u * stride;
            if (g < n) out[g] = a[u] + b[u];
        }
    }
}

// the preconditioner of the flexible solver: the network, the background
// solve, or the two composed (compose: 0 background then network on its
// residual, 1 network then background on its residual, 2 background, network,
// background)
struct Precond {
    bella_cnn *net;
    bella_spectral3d *sp;
    int compose;
};

// out += correction of the stage that maps the residual in - A out; c1/c2 scratch
static int stage_net(bella_ws *ws, const Precond &pc, const float *in, float *out, cudaStream_t s) {
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    float *tmp = spectral_work(pc.sp, 0), *corr = spectral_work(pc.sp, 1);
    op_apply(ws, 1, out, tmp, s);
    k_flex_corr_in<<<gv, VEC_BLOCK, 0, s>>>(n, in, tmp, ws->ks, ws->partials, ws->counter);
    const int rc = cnn_apply_dev(pc.net, ws->nx, ws->ny, ws->nz, tmp, corr, &ws->ks->pss, s, ws->per);
    if (rc != BELLA_OK) return set_err(rc, "bella_fbicgstab_pc: grid exceeds the network's capacity");
    k_flex_add<<<gv, VEC_BLOCK, 0, s>>>(n, out, corr, ws->ks);
    ws->launches += 3;
    return BELLA_OK;
}

static int stage_background(bella_ws *ws, const Precond &pc, const float *in, float *out, cudaStream_t s) {
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    float *tmp = spectral_work(pc.sp, 0), *corr = spectral_work(pc.sp, 1);
    op_apply(ws, 1, out, tmp, s);
    k_flex_corr_in<<<gv, VEC_BLOCK, 0, s>>>(n, in, tmp, ws->ks, ws->partials, ws->counter);
    int rc = spectral_apply_dev(pc.sp, tmp, corr, s);
    if (rc != BELLA_OK) return cuda_check(cudaGetLastError(), "bella_fbicgstab_pc: background solve");
    k_flex_add<<<gv, VEC_BLOCK, 0, s>>>(n, out, corr, ws->ks);
    ws->launches += 3;
    return BELLA_OK;
}

static int precond_apply(bella_ws *ws, const Precond &pc, const float *in, float *out, double *in_sumsq,
                         cudaStream_t s) {
    if (!pc.sp) {
        // the network alone: no seam band left out (there is no other stage to cover it)
        const int rc = cnn_apply_dev(pc.net, ws->nx, ws->ny, ws->nz, in, out, in_sumsq, s);
        if (rc != BELLA_OK) return set_err(rc, "bella_fbicgstab: grid exceeds the network's capacity");
        return BELLA_OK;
    }
    int rc;
    if (pc.net && pc.compose == 1) {
        rc = cnn_apply_dev(pc.net, ws->nx, ws->ny, ws->nz, in, out, in_sumsq, s, ws->per);
        if (rc != BELLA_OK) return set_err(rc, "bella_fbicgstab_pc: grid exceeds the network's capacity");
        return stage_background(ws, pc, in, out, s);
    }
    rc = spectral_apply_dev(pc.sp, in, out, s);
    if (rc != BELLA_OK) return cuda_check(cudaGetLastError(), "bella_fbicgstab_pc: background solve");
    if (!pc.net) return BELLA_OK;
    rc = stage_net(ws, pc, in, out, s);
    if (rc != BELLA_OK || pc.compose != 2) return rc;
    return stage_background(ws, pc, in, out, s);
}

static int flex_iteration(bella_ws *ws, const Precond &pc, cudaStream_t s) {
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    double *scale = &ws->ks->dot_aux;   // device address of the running sum of squares
    k_flex_p<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r32, ws->p32[0], ws->v32[0], ws->ks, ws->partials, ws->counter);
    int rc = precond_apply(ws, pc, ws->p32[0], ws->ph32, scale, s);
    if (rc != BELLA_OK) return rc;
    op_apply(ws, 1, ws->ph32, ws->v32[0], s);
    k_flex_alpha<<<gv, VEC_BLOCK, 0, s>>>(n, ws->rh32, ws->v32[0], ws->ks, ws->partials, ws->counter);
    k_flex_s<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r32, ws->v32[0], ws->s32, ws->ks, ws->partials, ws->counter);
    rc = precond_apply(ws, pc, ws->s32, ws->sh32, scale, s);
    if (rc != BELLA_OK) return rc;
    op_apply(ws, 1, ws->sh32, ws->t32, s);
    k_flex_omega<<<gv, VEC_BLOCK, 0, s>>>(n, ws->t32, ws->s32, ws->ks, ws->partials, ws->counter);
    k_flex_update<<<gv, VEC_BLOCK, 0, s>>>(n, ws->x32, ws->ph32, ws->sh32, ws->r32, ws->s32, ws->t32, ws->rh32,
                                           ws->ks, ws->partials, ws->counter);
    ws->launches += 7;
    return cuda_check(cudaGetLastError(), "flexible BiCGStab iteration");
}

static int run_flex(bella_ws *ws, const Precond &pc, const bella_solve_opts *o, cudaStream_t s,
                    std::chrono::steady_clock::time_point t0, int *timed_out) {
    const int blk = o->check_every > 0 ? (o->check_every < 4 ? o->check_every : 4) : 4;
    *timed_out = 0;
    for (;;) {
        int rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        if (ws->ks_host->done) return BELLA_OK;
        if (o->timeout_s > 0.0) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el > o->timeout_s) { *timed_out = 1; return BELLA_OK; }
        }
        for (int k = 0; k < blk; ++k) {
            rc = flex_iteration(ws, pc, s);
            if (rc != BELLA_OK) return rc;
        }
    }
}

// ---------------------------------------------------------------------------
// Flexible GMRES (Saad's FGMRES): the inner solver for preconditioners that are
// not one fixed linear map (the BF16 network).  One cycle of up to m
// iterations per refinement step; Arnoldi vectors in FP32, every inner product
// in FP64, classical Gram-Schmidt with one reorthogonalisation pass; the small
// Hessenberg least-squares problem (Givens rotations) on the host.
// ---------------------------------------------------------------------------
constexpr int FG_MAXM = 64;
constexpr int FG_MAXV = FG_MAXM + 1;

// blocks of the Gram-Schmidt kernels: 4 per SM, one resident wave (at 40-52
// registers a thread 4-6 blocks of 256 fit an SM; 8 per SM ran a second, partial
// wave that cost ~10 us a launch: 41 -> 30 us for the inner products with one
// basis vector at 257x129x257)
static int fg_xblk() { return num_sms() * 4; }
constexpr int FG_GROUP = 8;         // inner products per block

// The Arnoldi vectors are columns of leading dimension fg_ld(n), a multiple of 4,
// so every column starts on a 16-byte boundary: the Gram-Schmidt kernels read
// four consecutive elements at a time (float4), the n mod 4 last ones in block 0.
__device__ __forceinline__ float4 ld4(const float *p, long long i4) { return reinterpret_cast<const float4 *>(p)[i4]; }
__device__ __forceinline__ void st4(float *p, long long i4, float4 v) { reinterpret_cast<float4 *>(p)[i4] = v; }

// block (bx, gy): partial sums of <V_i, w> for the FG_GROUP vectors i of group gy
// over a grid-stride share -> part[i * gridDim.x + bx]; w is read once per group.
// With FG_XBLK x 256 threads each thread adds a few tens of products (FP32, on
// the FP32 pipe); block and grid sums are FP64.
__global__ void __launch_bounds__(VEC_BLOCK)
k_fg_mdot(long long n, const float *__restrict__ V, long long ld, int nv, const float *__restrict__ w,
          double *__restrict__ part) {
    const int i0 = blockIdx.y * FG_GROUP;
    const int cnt = nv - i0 < FG_GROUP ? nv - i0 : FG_GROUP;
    float acc[FG_GROUP];
#pragma unroll
    for (int q = 0; q < FG_GROUP; ++q) acc[q] = 0.f;
    const long long n4 = n >> 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 wv = ld4(w, i);
        float4 v[FG_GROUP];                           // every vector's load issued before the products
#pragma unroll
        for (int q = 0; q < FG_GROUP; ++q) v[q] = q < cnt ? ld4(V + (i0 + q) * ld, i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int q = 0; q < FG_GROUP; ++q) {
            acc[q] = fmaf(v[q].x, wv.x, acc[q]);
            acc[q] = fmaf(v[q].y, wv.y, acc[q]);
            acc[q] = fmaf(v[q].z, wv.z, acc[q]);
            acc[q] = fmaf(v[q].w, wv.w, acc[q]);
        }
    }
    if (blockIdx.x == 0)
        for (long long g = 4 * n4 + threadIdx.x; g < n; g += blockDim.x) {
            const float wg = w[g];
#pragma unroll
            for (int q = 0; q < FG_GROUP; ++q)
                if (q < cnt) acc[q] = fmaf(V[(i0 + q) * ld + g], wg, acc[q]);
        }
    __shared__ double red[FG_GROUP][VEC_BLOCK / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < FG_GROUP; ++q) {
        const double v = warp_sum((double)acc[q]);
        if (lane == 0) red[q][wid] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
        double sum = 0.0;
        for (int k = 0; k < VEC_BLOCK / 32; ++k) sum += red[threadIdx.x][k];
        part[(size_t)(i0 + threadIdx.x) * gridDim.x + blockIdx.x] = sum;
    }
}

// out[q] = sum over blocks of part[q * nblk + b]: block q, fixed strided partial
// sums and a fixed tree (deterministic)
__global__ void __launch_bounds__(256) k_fg_reduce(int nblk, const double *part, int nq, double *out) {
    const int q = blockIdx.x;
    if (q >= nq) return;
    double sum = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) sum += part[(size_t)q * nblk + b];
    __shared__ double red[256];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[q] = red[0];
}

// w -= sum_i h[i] V_i, and with norm per-block partial sums of the new <w, w> (slot 0)
__global__ void __launch_bounds__(VEC_BLOCK)
k_fg_update(long long n, const float *__restrict__ V, long long ld, int nv, const double *__restrict__ h,
            float *__restrict__ w, int norm, double *__restrict__ part) {
    __shared__ float hs[FG_MAXV];
    if ((int)threadIdx.x < nv) hs[threadIdx.x] = (float)h[threadIdx.x];
    __syncthreads();
    DF acc;
    acc.zero();
    const long long n4 = n >> 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        float4 wv = ld4(w, i);
        for (int q = 0; q < nv; ++q) {
            const float4 v = ld4(V + q * ld, i);
            const float hq = -hs[q];
            wv.x = fmaf(hq, v.x, wv.x);
            wv.y = fmaf(hq, v.y, wv.y);
            wv.z = fmaf(hq, v.z, wv.z);
            wv.w = fmaf(hq, v.w, wv.w);
        }
        st4(w, i, wv);
        if (norm) {
            acc.add_prod(wv.x, wv.x);
            acc.add_prod(wv.y, wv.y);
            acc.add_prod(wv.z, wv.z);
            acc.add_prod(wv.w, wv.w);
        }
    }
    if (blockIdx.x == 0)
        for (long long g = 4 * n4 + threadIdx.x; g < n; g += blockDim.x) {
            float wg = w[g];
            for (int q = 0; q < nv; ++q) wg = fmaf(-hs[q], V[q * ld + g], wg);
            w[g] = wg;
            if (norm) acc.add_prod(wg, wg);
        }
    if (!norm) return;
    __shared__ double red[VEC_BLOCK / 32];
    const double v = warp_sum(acc.value());
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int k = 0; k < VEC_BLOCK / 32; ++k) sum += red[k];
        part[blockIdx.x] = sum;
    }
}

// out = w / sqrt(*nrm2) (in place allowed); zero when the norm is not positive;
// both 16-byte aligned (Arnoldi columns, the workspace's r32)
__global__ void k_fg_scale(long long n, const float *w, const double *nrm2, float *out) {
    const double q = *nrm2;
    const float inv = (q > 0.0 && isfinite(q)) ? (float)(1.0 / sqrt(q)) : 0.f;
    const long long n4 = n >> 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 v = ld4(w, i);
        st4(out, i, make_float4(v.x * inv, v.y * inv, v.z * inv, v.w * inv));
    }
    if (blockIdx.x == 0)
        for (long long g = 4 * n4 + threadIdx.x; g < n; g += blockDim.x) out[g] = w[g] * inv;
}

// x += sum_i y[i] Z_i (x: the workspace's x32, 16-byte aligned)
__global__ void k_fg_combine(long long n, const float *Z, long long ld, int nz, const double *y, float *x) {
    __shared__ float ys[FG_MAXM];
    if ((int)threadIdx.x < nz) ys[threadIdx.x] = (float)y[threadIdx.x];
    __syncthreads();
    const long long n4 = n >> 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        float4 xv = ld4(x, i);
        for (int q = 0; q < nz; ++q) {
            const float4 v = ld4(Z + q * ld, i);
            xv.x = fmaf(ys[q], v.x, xv.x);
            xv.y = fmaf(ys[q], v.y, xv.y);
            xv.z = fmaf(ys[q], v.z, xv.z);
            xv.w = fmaf(ys[q], v.w, xv.w);
        }
        st4(x, i, xv);
    }
    if (blockIdx.x == 0)
        for (long long g = 4 * n4 + threadIdx.x; g < n; g += blockDim.x) {
            float xg = x[g];
            for (int q = 0; q < nz; ++q) xg = fmaf(ys[q], Z[q * ld + g], xg);
            x[g] = xg;
        }
}

// leading dimension of the Arnoldi columns: n rounded up to a multiple of 4
static long long fg_ld(long long n) { return (n + 3) & ~3LL; }

static int fg_ensure(bella_ws *ws, int m) {
    const long long n = ws->n;
    if (ws->fg_v && ws->fg_m >= m && ws->fg_n == n) return BELLA_OK;
    cudaFree(ws->fg_v); cudaFree(ws->fg_z); cudaFree(ws->fg_part); cudaFree(ws->fg_dev);
    ws->fg_v = ws->fg_z = nullptr;
    ws->fg_part = ws->fg_dev = nullptr;
    ws->fg_m = 0;
    BELLA_CUDA(cudaMalloc(&ws->fg_v, (size_t)(m + 1) * fg_ld(n) * sizeof(float)));
    BELLA_CUDA(cudaMalloc(&ws->fg_z, (size_t)m * fg_ld(n) * sizeof(float)));
    BELLA_CUDA(cudaMalloc(&ws->fg_part, (size_t)MAXGRID * (FG_MAXV + 1) *
                                        sizeof(double)));
    BELLA_CUDA(cudaMalloc(&ws->fg_dev, 4 * (FG_MAXV + 1) * sizeof(double)));
    const double one = 1.0;
    BELLA_CUDA(cudaMemcpy(ws->fg_dev + 3 * (FG_MAXV + 1), &one, sizeof(double), cudaMemcpyHostToDevice));
    ws->fg_m = m;
    ws->fg_n = n;
    return BELLA_OK;
}

// One FGMRES cycle on A x32 = r32 (x32 = 0 on entry, r32 = the scaled outer
// residual set by k_init32, ||r32||^2 in ks->rr): stops when the Arnoldi
// residual estimate falls to rel*||r32|| or after m iterations.  *iters gets
// the iterations, *status BELLA_OK / BELLA_MAXITER / BELLA_NONFINITE.
static int fgmres_cycle(bella_ws *ws, const Precond &pc, int m, double rel, cudaStream_t s, int *iters,
                        int *status) {
    const long long n = ws->n;
    const int gv = fg_xblk();                          // one resident wave (see fg_xblk)
    double *h1 = ws->fg_dev, *h2 = ws->fg_dev + (FG_MAXV + 1), *nrm = ws->fg_dev + 2 * (FG_MAXV + 1);
    double *unit = ws->fg_dev + 3 * (FG_MAXV + 1);   // 1.0: sum of squares of a basis vector
    float *V = ws->fg_v, *Z = ws->fg_z;
    const long long ld = fg_ld(n);
    int rc = sync_state(ws, s);
    if (rc != BELLA_OK) return rc;
    const double beta = sqrt(ws->ks_host->rr);
    *iters = 0;
    *status = BELLA_MAXITER;
    if (!isfinite(beta)) { *status = BELLA_NONFINITE; return BELLA_OK; }
    if (!(beta > 0.0)) { *status = BELLA_OK; return BELLA_OK; }
    k_fg_scale<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r32, &ws->ks->rr, V);
    const int xb = fg_xblk();
    double H[FG_MAXV][FG_MAXM], cs[FG_MAXM], sn[FG_MAXM], gvec[FG_MAXV];
    memset(H, 0, sizeof(H));
    gvec[0] = beta;
    double hhost[3 * (FG_MAXV + 1)];
    int j = 0, k = 0;
    for (j = 0; j < m; ++j) {
        float *vj = V + (size_t)j * ld, *zj = Z + (size_t)j * ld, *w = V + (size_t)(j + 1) * ld;
        rc = precond_apply(ws, pc, vj, zj, unit, s);
        if (rc != BELLA_OK) return rc;
        op_apply(ws, 1, zj, w, s);
        const int nv = j + 1;
        const unsigned ng = (unsigned)((nv + FG_GROUP - 1) / FG_GROUP);
        k_fg_mdot<<<dim3(xb, ng), VEC_BLOCK, 0, s>>>(n, V, ld, nv, w, ws->fg_part);
        k_fg_reduce<<<nv, 256, 0, s>>>(xb, ws->fg_part, nv, h1);
        k_fg_update<<<gv, VEC_BLOCK, 0, s>>>(n, V, ld, nv, h1, w, 0, ws->fg_part);
        k_fg_mdot<<<dim3(xb, ng), VEC_BLOCK, 0, s>>>(n, V, ld, nv, w, ws->fg_part);
        k_fg_reduce<<<nv, 256, 0, s>>>(xb, ws->fg_part, nv, h2);
        k_fg_update<<<gv, VEC_BLOCK, 0, s>>>(n, V, ld, nv, h2, w, 1, ws->fg_part);
        k_fg_reduce<<<1, 256, 0, s>>>(gv, ws->fg_part, 1, nrm);
        k_fg_scale<<<gv, VEC_BLOCK, 0, s>>>(n, w, nrm, w);
        ws->launches += 10;
        BELLA_CUDA(cudaMemcpyAsync(hhost, ws->fg_dev, sizeof(hhost), cudaMemcpyDeviceToHost, s));
        BELLA_CUDA(cudaStreamSynchronize(s));
        BELLA_CUDA(cudaGetLastError());
        for (int i = 0; i <= j; ++i) H[i][j] = hhost[i] + hhost[(FG_MAXV + 1) + i];
        H[j + 1][j] = sqrt(fmax(hhost[2 * (FG_MAXV + 1)], 0.0));
        bool finite = isfinite(H[j + 1][j]);
        for (int i = 0; i <= j; ++i) finite = finite && isfinite(H[i][j]);
        if (!finite) { *status = BELLA_NONFINITE; *iters = j + 1; return BELLA_OK; }
        for (int i = 0; i < j; ++i) {             // earlier rotations
            const double t = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
            H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
            H[i][j] = t;
        }
        const double a = H[j][j], b = H[j + 1][j];
        const double r = hypot(a, b);
        cs[j] = r > 0.0 ? a / r : 1.0;
        sn[j] = r > 0.0 ? b / r : 0.0;
        H[j][j] = r;
        H[j + 1][j] = 0.0;
        gvec[j + 1] = -sn[j] * gvec[j];
        gvec[j] = cs[j] * gvec[j];
        k = j + 1;
        if (fabs(gvec[j + 1]) <= rel * beta) { *status = BELLA_OK; break; }
        if (b == 0.0) { *status = BELLA_OK; break; }   // invariant subspace: exact in it
    }
    // y = H^-1 g (upper triangular k x k), x32 = Z y
    double y[FG_MAXM];
    for (int i = k - 1; i >= 0; --i) {
        double t = gvec[i];
        for (int l = i + 1; l < k; ++l) t -= H[i][l] * y[l];
        y[i] = H[i][i] != 0.0 ? t / H[i][i] : 0.0;
    }
    BELLA_CUDA(cudaMemcpyAsync(ws->fg_dev, y, k * sizeof(double), cudaMemcpyHostToDevice, s));
    k_fg_combine<<<gv, VEC_BLOCK, 0, s>>>(n, Z, ld, k, ws->fg_dev, ws->x32);
    ws->launches += 1;
    BELLA_CUDA(cudaStreamSynchronize(s));   // y lives on this stack frame until the copy is done
    *iters = k;
    return cuda_check(cudaGetLastError(), "flexible GMRES cycle");
}

}  // namespace bella

static int fbicgstab_impl(bella_ws *ws, const bella::Precond &pc, const double *b, double *x,
                          const bella_solve_opts *opts, bella_solve_stats *stats, void *stream,
                          int restart = 0) {
    if (ws->ndim == 0) return set_err(BELLA_ENOOP, "bella_fbicgstab: no operator set");
    if (pc.net && ws->ndim != 3)
        return set_err(BELLA_EINVAL, "bella_fbicgstab: the network needs a 3D operator (bella_op3d_set)");
    bella_solve_opts o;
    if (opts) o = *opts; else bella_solve_opts_default(&o);
    if (!(o.tol >= 0.0) || o.maxiter < 0) return set_err(BELLA_EINVAL, "bella_fbicgstab: bad tol/maxiter");
    BELLA_CUDA(cudaSetDevice(ws->device));
    cudaStream_t s = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    // the refinement's residuals b - A x: in double-float arithmetic on a 3D operator when
    // the tolerance leaves room for its rounding (about 1e-14 of |A||x|; GB300's FP64 pipe
    // makes the FP64 stencil twice as slow), in FP64 otherwise
    const bool df_resid = ws->ndim == 3 && o.tol >= 1e-11;
    auto refine_resid = [&]() {
        if (df_resid) op3d_resid_df(ws, x, b, ws->r64, s);
        else op_resid(ws, 0, x, b, ws->r64, s);
    };
    bella_solve_stats st;
    memset(&st, 0, sizeof(st));
    const long long n = ws->n;
    const int gv = ws->grid_vec;
    int rc, timed_out = 0;
    k_dot64<<<gv, VEC_BLOCK, 0, s>>>(n, b, b, ws->ks, ws->partials, ws->counter);
    ws->launches++;
    rc = sync_state(ws, s);
    if (rc != BELLA_OK) return rc;
    const double bnorm = sqrt(ws->ks_host->dot_aux);
    st.bnorm = bnorm;
    double target = o.tol * bnorm;
    if (o.atol > target) target = o.atol;
    bool failed = false;
    double rn_known = -1.0;                           // >= 0: ||b - A x|| of the current x, measured
    if (!isfinite(bnorm)) {
        st.status = BELLA_NONFINITE;
    } else if (o.x0_zero && (bnorm == 0.0 || bnorm <= o.tol)) {   // scipy 1.7 legacy exit
        BELLA_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        st.status = BELLA_OK;
    } else {
        NullSpace ns = ws->ns;
        if (!o.project_null) ns.nm = 0;
        double rnorm = bnorm;
        if (o.x0_zero) {                              // r = b - A 0 = b exactly: no stencil
            BELLA_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
            BELLA_CUDA(cudaMemcpyAsync(ws->r64, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        } else {
            refine_resid();
            rc = sync_state(ws, s);
            if (rc != BELLA_OK) return rc;
            rnorm = sqrt(ws->ks_host->dot_aux2);
            st.matvecs = 1;
        }
        int total = 0;
        for (int outer = 0;; ++outer) {
            if (!isfinite(rnorm)) { st.status = BELLA_NONFINITE; failed = true; break; }
            if (rnorm <= target) { st.status = BELLA_OK; break; }
            if (total >= o.maxiter) { st.status = BELLA_MAXITER; break; }
            if (outer >= o.max_outer) { failed = true; break; }
            if (timed_out) { st.status = BELLA_TIMEOUT; break; }
            double rel = o.inner_tol;
            const double need = 0.5 * target / rnorm;
            if (need > rel) rel = need;
            // each inner solve is capped so that a stagnating learned iteration is
            // checked (and, without progress, replaced by the plain method) early
            int cap = o.maxiter / (o.max_outer > 0 ? o.max_outer : 1);
            if (cap < 100) cap = 100;
            if (cap > o.maxiter - total) cap = o.maxiter - total;
            k_init32<<<gv, VEC_BLOCK, 0, s>>>(n, ws->r64, 1.0 / rnorm, ws->r32, ws->rh32, ws->x32, rel, cap, ws->ks,
                                              ws->partials, ws->counter);
            ws->launches++;
            int it, inner_status;
            if (restart > 0) {
                rc = fgmres_cycle(ws, pc, restart < cap ? restart : cap, rel, s, &it, &inner_status);
                if (rc != BELLA_OK) return rc;
                if (o.timeout_s > 0.0 &&
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > o.timeout_s)
                    timed_out = 1;
            } else {
                rc = run_flex(ws, pc, &o, s, t0, &timed_out);
                if (rc != BELLA_OK) return rc;
                it = ws->ks_host->iter;
                inner_status = ws->ks_host->status;
                st.detail = ws->ks_host->pad[0];
            }
            total += it;
            st.matvecs += (restart > 0 ? 1 : 2) * it;
            st.outer = outer + 1;
            if (inner_status == BELLA_NONFINITE || it == 0) { failed = true; break; }
            BELLA_CUDA(cudaMemcpyAsync(ws->x64v, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            k_ir_update<<<gv, VEC_BLOCK, 0, s>>>(n, x, ws->x32, rnorm, ws->z64, ns, ws->ks, ws->partials,
                                                 ws->counter);
            ws->launches++;
            if (ns.nm > 0) {   // range projection before the residual is measured (as in the plain loop)
                k_null_shift<<<gv, VEC_BLOCK, 0, s>>>(n, x, ws->ks, ns);
                ws->launches++;
            }
            refine_resid();
            st.matvecs += 1;
            rc = sync_state(ws, s);
            if (rc != BELLA_OK) return rc;
            const double rnew = sqrt(ws->ks_host->dot_aux2);
            if (!(rnew < rnorm)) {   // no progress: restore the iterate, fall back
                BELLA_CUDA(cudaMemcpyAsync(x, ws->x64v, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                failed = true;
                break;
            }
            rnorm = rnew;
        }
        st.iterations = total;
        if (failed) {
            // the plain method from the current iterate; reported, never silent
            st.fallback = 1;
            const int left = o.maxiter - total;
            bella_solve_stats fs;
            memset(&fs, 0, sizeof(fs));
            rc = solve_df(ws, b, x, o, 1, left > 0 ? left : 0, &fs, s, t0);
            if (rc != BELLA_OK) return rc;
            st.status = fs.status;
            st.iterations += fs.iterations;
            st.matvecs += fs.matvecs;
            st.detail = fs.detail;
        } else {
            rn_known = rnorm;                         // the loop measured the returned x's residual last
        }
    }
    double rn = rn_known;
    if (!(rn >= 0.0)) {                               // true FP64 residual of the returned x
        op_resid(ws, 0, x, b, ws->r64, s);
        rc = sync_state(ws, s);
        if (rc != BELLA_OK) return rc;
        rn = sqrt(ws->ks_host->dot_aux2);
    }
    st.relres = st.bnorm > 0 ? rn / st.bnorm : rn;
    if (!isfinite(rn)) st.status = BELLA_NONFINITE;
    BELLA_CUDA(cudaGetLastError());
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return st.status;
}

extern "C" int bella_fbicgstab(bella_ws *ws, bella_cnn *net, const double *b, double *x,
                               const bella_solve_opts *opts, bella_solve_stats *stats, void *stream) {
    if (!ws || !net || !b || !x) return set_err(BELLA_EINVAL, "bella_fbicgstab: null argument");
    return fbicgstab_impl(ws, bella::Precond{net, nullptr, 0}, b, x, opts, stats, stream);
}

extern "C" int bella_fbicgstab_pc(bella_ws *ws, bella_spectral3d *sp, bella_cnn *net, int compose, const double *b,
                                  double *x, const bella_solve_opts *opts, bella_solve_stats *stats, void *stream) {
    if (!ws || (!sp && !net) || !b || !x) return set_err(BELLA_EINVAL, "bella_fbicgstab_pc: null argument");
    if (compose < 0 || compose > 2) return set_err(BELLA_EINVAL, "bella_fbicgstab_pc: compose must be 0, 1 or 2");
    if (sp && bella::spectral_size(sp) != ws->n)
        return set_err(BELLA_EINVAL, "bella_fbicgstab_pc: background solve made for another grid");
    return fbicgstab_impl(ws, bella::Precond{net, sp, compose}, b, x, opts, stats, stream);
}

extern "C" int bella_fgmres_pc(bella_ws *ws, bella_spectral3d *sp, bella_cnn *net, int compose, int restart,
                               const double *b, double *x, const bella_solve_opts *opts, bella_solve_stats *stats,
                               void *stream) {
    if (!ws || (!sp && !net) || !b || !x) return set_err(BELLA_EINVAL, "bella_fgmres_pc: null argument");
    if (compose < 0 || compose > 2) return set_err(BELLA_EINVAL, "bella_fgmres_pc: compose must be 0, 1 or 2");
    if (restart < 1 || restart > bella::FG_MAXM) return set_err(BELLA_EINVAL, "bella_fgmres_pc: restart must be 1..64");
    if (ws->ndim == 0) return set_err(BELLA_ENOOP, "bella_fgmres_pc: no operator set");
    if (sp && bella::spectral_size(sp) != ws->n)
        return set_err(BELLA_EINVAL, "bella_fgmres_pc: background solve made for another grid");
    BELLA_CUDA(cudaSetDevice(ws->device));
    int rc = bella::fg_ensure(ws, restart);
    if (rc != BELLA_OK) return rc;
    return fbicgstab_impl(ws, bella::Precond{net, sp, compose}, b, x, opts, stats, stream, restart);
}

// ============================================================================
// Allocation-free FP64 BiCGStab for small 2D systems.
//
// Some callers cannot allocate device memory while they run: a model that
// reserves the whole GPU for its own memory pool at start-up and forbids any
// later cudaMalloc, or a time loop that cannot afford the device-wide
// synchronisation a cudaMalloc/cudaFree may cause.  For them this entry point
// keeps every byte of its scratch (packed operator planes, Krylov vectors,
// reduction partials, Krylov state) in one file-scope device array of fixed
// size, created when the library's device code is loaded on a GPU and held by
// every GPU that loads the library until the process exits.
// ============================================================================
#include <mutex>

namespace bella {

constexpr long long NOALLOC_MAX_NODES = 65536;                   // nx*ny
constexpr long long NOALLOC_MAX_CELLS = 2 * NOALLOC_MAX_NODES;   // (nx+1)*(ny+1)
constexpr long long NOALLOC_PARTIALS = (long long)NQ * MAXGRID;
// doubles: 4 FP64 cell planes + 4 FP32 cell planes (as 2 doubles' worth),
// dinv/hc/z (FP64) + dinv/hc (FP32, one double's worth), 9 FP64 vectors,
// partials, counter word and the Krylov state
constexpr long long NOALLOC_DOUBLES =
    6 * NOALLOC_MAX_CELLS + 4 * NOALLOC_MAX_NODES + 9 * NOALLOC_MAX_NODES + NOALLOC_PARTIALS + 8 +
    (long long)((sizeof(KState) + 7) / 8);

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[256];   // device address of g_noalloc_scratch per device

// Device address of the scratch array on the current device (looked up once
// per device with that device current; the array's host-side name is not a
// device address).
static int noalloc_scratch(int dev, double **out) {
    if (dev < 0 || dev >= 256) return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: device id out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return BELLA_OK;
}

}  // namespace bella

extern "C" int bella_bicgstab2d_noalloc(const bella_op2d *op, const double *b, double *x,
                                        const bella_solve_opts *opts, bella_solve_stats *stats,
                                        void *stream) {
    using namespace bella;
    if (!op || !b || !x) return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: null argument");
    if (op->nx < 3 || op->ny < 3) return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: nx, ny must be >= 3");
    const long long n = (long long)op->nx * op->ny;
    const long long nc = (long long)(op->nx + 1) * (op->ny + 1);
    if (n > NOALLOC_MAX_NODES || nc > NOALLOC_MAX_CELLS)
        return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: grid too large for the fixed scratch "
                                     "(at most 65536 nodes and 131072 cells); use bella_bicgstab");
    if (!op->hplusx || !op->hplusy || !op->cxx || !op->cyy || !op->diag_inv)
        return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: hplusx, hplusy, cxx, cyy, diag_inv are required");
    if (op->x_wall < 0 || op->x_wall > 1 || op->y_wall < 0 || op->y_wall > 1)
        return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: x_wall, y_wall must be 0 or 1");
    if (!(op->dx > 0.0) || !(op->dy > 0.0)) return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: dx, dy must be > 0");
    bella_solve_opts o;
    if (opts) {
        o = *opts;
    } else {   // the shared defaults, with the one precision this entry point has
        bella_solve_opts_default(&o);
        o.precision = 0;
    }
    if (!(o.tol >= 0.0) || o.maxiter < 0) return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: bad tol/maxiter");
    if (o.precision != 0)
        return set_err(BELLA_EINVAL, "bella_bicgstab2d_noalloc: only precision 0 (FP64 BiCGStab) is available");
    int dev = 0;
    BELLA_CUDA(cudaGetDevice(&dev));
    double *base = nullptr;
    int rc = noalloc_scratch(dev, &base);
    if (rc != BELLA_OK) return rc;

    // a workspace view onto the fixed scratch; lives on this call's stack
    bella_ws w;
    memset(&w, 0, sizeof(w));
    KState ks_host;
    w.device = dev;
    w.ndim = 2;
    w.nx = op->nx; w.ny = op->ny; w.nz = 1;
    w.n = n;
    w.cross = (op->cxy != nullptr || op->cyx != nullptr) ? 1 : 0;
    w.has_hc = op->hcenter != nullptr ? 1 : 0;
    w.singular = 0;            // no null-space projection on the FP64 path
    w.grid_stencil = stencil_grid(op->nx, op->ny);
    w.grid_vec = vec_grid(n);
    double *p = base;
    w.a64 = p;                 p += 4 * NOALLOC_MAX_CELLS;
    w.a32 = (float *)p;        p += 2 * NOALLOC_MAX_CELLS;
    w.dinv64 = p;              p += NOALLOC_MAX_NODES;
    w.hc64 = p;                p += NOALLOC_MAX_NODES;
    w.z64 = p;                 p += NOALLOC_MAX_NODES;
    w.dinv32 = (float *)p;     // dinv32 and hc32 share one slab of MAX_NODES doubles
    w.hc32 = w.dinv32 + NOALLOC_MAX_NODES;
    p += NOALLOC_MAX_NODES;
    w.r64 = p;                 p += NOALLOC_MAX_NODES;
    w.x64v = p;                p += NOALLOC_MAX_NODES;
    w.r64k = p;                p += NOALLOC_MAX_NODES;
    w.rh64 = p;                p += NOALLOC_MAX_NODES;
    w.p64[0] = p;              p += NOALLOC_MAX_NODES;
    w.p64[1] = p;              p += NOALLOC_MAX_NODES;
    w.v64[0] = p;              p += NOALLOC_MAX_NODES;
    w.v64[1] = p;              p += NOALLOC_MAX_NODES;
    w.t64 = p;                 p += NOALLOC_MAX_NODES;
    w.partials = p;            p += NOALLOC_PARTIALS;
    w.counter = (unsigned *)p; p += 8;
    w.ks = (KState *)p;
    w.ks_host = &ks_host;
    w.cap = n;

    cudaStream_t s = (cudaStream_t)stream;
    const auto t0 = std::chrono::steady_clock::now();
    // the array keeps the previous call's contents: the grid-reduction counter
    // must start at zero
    BELLA_CUDA(cudaMemsetAsync(w.counter, 0, 8 * sizeof(double), s));
    rc = op2d_pack(&w, op, s);
    if (rc != BELLA_OK) return cuda_check(cudaGetLastError(), "bella_bicgstab2d_noalloc: pack");
    bella_solve_stats st;
    memset(&st, 0, sizeof(st));
    rc = solve_fp64(&w, b, x, o, o.x0_zero ? 0 : 1, o.maxiter, &st, s, t0);
    if (rc != BELLA_OK) return rc;
    op2d_resid(&w, 0, x, b, w.r64, s);
    rc = sync_state(&w, s);
    if (rc != BELLA_OK) return rc;
    const double rn = sqrt(ks_host.dot_aux2);
    st.relres = st.bnorm > 0 ? rn / st.bnorm : rn;
    if (!isfinite(rn)) st.status = BELLA_NONFINITE;
    BELLA_CUDA(cudaGetLastError());
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = st;
    return st.status;
}
