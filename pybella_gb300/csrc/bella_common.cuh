// bella_common.cuh -- shared device helpers and the workspace layout of
// libbella_gb300 (GB300 / sm_103a implicit nodal pressure projection).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/bella.h"
#include "bella_df.cuh"

namespace bella {

// --------------------------------------------------------------------------
// launch geometry of the 2D stencil tiles
// --------------------------------------------------------------------------
#ifndef BELLA_TY
#define BELLA_TY 16
#endif
#ifndef BELLA_MINB
#define BELLA_MINB 6            // measured best on GB300 (2049x1025, double-float: 57.6 us PDIR vs 63.0 at 5)
#endif
#ifndef BELLA_GRID_PER_SM
#define BELLA_GRID_PER_SM 8
#endif
constexpr int TX = 64;          // tile width  (nodes, x)  = 2 warps
constexpr int TY = BELLA_TY;    // tile height (nodes, y)
constexpr int MINB = BELLA_MINB;            // __launch_bounds__ min CTAs/SM of the stencil
constexpr int GRID_PER_SM = BELLA_GRID_PER_SM;
constexpr int BX = 64;          // threads in x
constexpr int BY = 4;           // threads in y  -> 256 threads, 4 rows each
constexpr int NTHREADS = BX * BY;
constexpr int MAX_SMS = 256;    // bound on the SM count: reduction partials are sized for MAX_SMS * 8 CTAs
int num_sms();                  // SM count of the current device (152 on GB300), queried once per device
constexpr int VEC_BLOCK = 256;  // block size of the streaming vector kernels
constexpr int NQ = 8;           // reduction quantities per kernel (max)
constexpr int MAXGRID = MAX_SMS * 8;  // largest grid of any reduction kernel (partials capacity)
constexpr int MAXNULL = 8;      // null-space modes handled by the projection

// --------------------------------------------------------------------------
// device-resident Krylov state.  Written only by the last block of a kernel
// (last-block-done reduction) and read by every block of the next kernel.
// --------------------------------------------------------------------------
struct KState {
    double rho;        // <r^, r> of the current residual
    double rho_prev;
    double alpha;
    double omega;
    double beta;
    double rr;         // ||r||^2
    double ss;         // ||s||^2
    double atol;       // absolute stopping threshold on ||r|| (and ||s||)
    double rhotol;     // rho / omega breakdown limit
    double rho0;       // <r^, r0>: scale of the relative rho breakdown test
    double scale;      // IR: inner system = outer residual / scale
    double dot_aux;    // result of the generic FP64 dot kernel
    double dot_aux2;
    double pss;        // sum of squares of the learned correction's input (flexible solver)
    int    iter;       // iterations done in this (inner) solve
    int    maxiter;    // iteration limit of this (inner) solve
    int    done;       // 1 once converged / failed: later kernels return at once
    int    status;     // BELLA_* status of the (inner) solve
    int    early;      // ||s|| < atol met inside the current iteration
    int    pad[3];     // pad[0]: breakdown reason (1 rho, 2 omega, 3 <r^,v>, 4 ||t||)
    double nd[MAXNULL];     // <z_k, x> of the null-space projection
    double cnull[MAXNULL];  // coefficients removed along the null modes
};

// --------------------------------------------------------------------------
// null space of the pseudo-incompressible operator (hcenter = 0, no cross
// terms): sign-pattern modes e(i,j,k) = sx^i sy^j sz^k (constants and the
// checkerboards the cell-averaged differences cannot see).  The left null
// vectors are z_k = D w e_k with D = 1/diag_inv and w the trapezoid weights
// (1/2 on a duplicated periodic seam).  ginv = inverse Gram matrix
// G_kl = <z_k, e_l>.
// --------------------------------------------------------------------------
struct NullSpace {
    int nm;
    int ndim, nx, ny, nz;
    signed char sx[MAXNULL], sy[MAXNULL], sz[MAXNULL];
    double ginv[MAXNULL * MAXNULL];
};

// parities of node g's grid indices (bit 0: i, bit 1: j, bit 2: k); 32-bit
// division (operators have fewer than 2^31 nodes: checked when they are set)
__device__ __forceinline__ int node_parity(const NullSpace &ns, long long g) {
    const unsigned gg = (unsigned)g;
    unsigned i, j, k;
    if (ns.ndim == 2) { j = gg / (unsigned)ns.nx; i = gg - j * (unsigned)ns.nx; k = 0u; }
    else {
        const unsigned t = gg / (unsigned)ns.nz;
        k = gg - t * (unsigned)ns.nz;
        i = t / (unsigned)ns.ny;
        j = t - i * (unsigned)ns.ny;
    }
    return (int)((i & 1u) | ((j & 1u) << 1) | ((k & 1u) << 2));
}

// value (+1 / -1) of null mode m at a node of parities p
__device__ __forceinline__ double null_mode_p(const NullSpace &ns, int m, int p) {
    int par = 0;
    if (ns.sx[m] < 0) par ^= p & 1;
    if (ns.sy[m] < 0) par ^= (p >> 1) & 1;
    if (ns.sz[m] < 0) par ^= (p >> 2) & 1;
    return par ? -1.0 : 1.0;
}

__device__ __forceinline__ double null_mode(const NullSpace &ns, int m, long long g) {
    return null_mode_p(ns, m, node_parity(ns, g));
}

// --------------------------------------------------------------------------
// double-float accumulation of FP32 products (error-free transformations):
// each product a*b = p + e exactly (fmaf), and the running sum keeps a
// compensated low word.  Converted to FP64 at the warp level, so the FP32
// Krylov inner products are accurate to ~1e-14 without per-element FP64
// arithmetic (GB300's FP64 pipe is narrow).
// --------------------------------------------------------------------------
struct DF {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = 0.f; lo = 0.f; }
    __device__ __forceinline__ void add_prod(float a, float b) {
        float p = a * b;
        float e = fmaf(a, b, -p);
        float s = hi + p;
        float bb = s - hi;
        float err = (hi - (s - bb)) + (p - bb);
        hi = s;
        lo += err + e;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

struct DD {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
    __device__ __forceinline__ double value() const { return v; }
};

template <typename T> struct Acc;
template <> struct Acc<float>  { using type = DF; };
template <> struct Acc<double> { using type = DD; };
template <> struct Acc<dfloat> { using type = DFAcc; };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NQ values (fixed tree order -> deterministic).  `red`
// must hold 32*NQ doubles of shared memory.  Result valid in thread 0.
template <int Q>
__device__ __forceinline__ void block_sum(double (&v)[Q], double *red) {
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nthreads = blockDim.x * blockDim.y;
    const int lane = tid & 31, wid = tid >> 5, nw = (nthreads + 31) >> 5;
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) red[wid * Q + q] = v[q];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) v[q] = (lane < nw) ? red[lane * Q + q] : 0.0;
#pragma unroll
        for (int q = 0; q < Q; ++q) v[q] = warp_sum(v[q]);
    }
    __syncthreads();
}

// Last-block-done grid reduction.  Every block writes its Q partial sums,
// the last block to arrive sums all partials in block order (deterministic)
// and returns true with the totals in `tot` (valid in every thread of that
// block).  `counter` is reset to 0 by the last block.
template <int Q>
__device__ __forceinline__ bool grid_sum(double (&v)[Q], double *partials, unsigned *counter,
                                         double (&tot)[Q]) {
    __shared__ double red[32 * NQ];
    __shared__ bool last;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int nthreads = blockDim.x * blockDim.y;
    block_sum<Q>(v, red);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) partials[(size_t)blockIdx.x * NQ + q] = v[q];
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) s[q] = 0.0;
    for (int b = tid; b < (int)gridDim.x; b += nthreads) {
#pragma unroll
        for (int q = 0; q < Q; ++q) s[q] += __ldcg(&partials[(size_t)b * NQ + q]);
    }
    block_sum<Q>(s, red);
    __shared__ double out[NQ];
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < Q; ++q) out[q] = s[q];
        *counter = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) tot[q] = out[q];
    return true;
}

// --------------------------------------------------------------------------
// prepared 2D operator (device pointers into the workspace)
//   cell planes (ny+1)*(nx+1): Axx = 0.5/dx^2 cxx hplusx, Ayy = 0.5/dy^2 cyy hplusy,
//   Axy = 0.5/(dx dy) cxy hplusy, Ayx = 0.5/(dx dy) cyx hplusx  (walls zeroed)
//   node planes ny*nx: dinv, hc
// --------------------------------------------------------------------------
template <typename T>
struct Op2D {
    int nx, ny;
    int ymirror;              // y boundary of the LAMB_BDRY stencil: node -1 <- node 1, node ny <- node ny-2
    const T *axx, *ayy, *axy, *ayx;
    const T *dinv, *hc;
};

}  // namespace bella

// --------------------------------------------------------------------------
// workspace (opaque to C callers)
// --------------------------------------------------------------------------
struct bella_ws {
    int device;
    int ndim;                 // 0: no operator yet
    // operator geometry (nz == 1 in 2D)
    int nx, ny, nz;
    long long n;              // unknowns
    int cross, has_hc, singular;
    int ymirror;              // 2D operator with the mirrored y boundary (bella_op2d.y_wall == BELLA_Y_MIRROR)
    int per[3];               // periodic axes of the operator (x, y, z; the duplicated seam)
    double *a64;              // 4 cell planes
    float  *a32;
    double *dinv64, *hc64, *z64;
    float  *dinv32, *hc32;
    bella::NullSpace ns;      // null modes (nm == 0: nonsingular)
    // Krylov storage
    long long cap;            // capacity (elements) of each vector below
    void *vbase;              // one allocation for all vectors
    double *r64, *x64v;       // IR outer residual, FP64 scratch
    float  *r32, *rh32, *p32[2], *v32[2], *t32, *x32;
    float  *s32, *ph32, *sh32;   // flexible (CNN-preconditioned) solver: s, M(p), M(s)
    double *r64k, *rh64, *p64[2], *v64[2], *t64;
    bella::dfloat *rdf, *rhdf, *pdf[2], *vdf[2], *tdf, *xdf;   // double-float Krylov vectors
    bella::dfloat *adf, *dinvdf, *hcdf;                         // double-float operator planes
    double *partials;
    unsigned *counter;
    bella::KState *ks;        // device
    bella::KState *ks_host;   // pinned mirror
    int grid_stencil, grid_vec;
    long long launches;
    // flexible GMRES: Arnoldi basis V [(m+1)][n], preconditioned basis Z [m][n],
    // per-block partial dot products and small device results
    float *fg_v, *fg_z;
    double *fg_part, *fg_dev;
    int fg_m;
    long long fg_n;
    // scratch of the device projection (bella_projection2d)
    double *proj_buf;
    size_t proj_cap;
    // the background solve of the device projections, kept between calls and
    // re-derived in place from each call's coefficients
    bella_spectral3d *sp_cache;
    // optional per-kernel timing with CUDA events (bella_ws_profile)
    int prof;
    struct Prof {
        cudaEvent_t ev[2 * 256];
        int pending;            // recorded pairs not yet harvested
        double total_ms;
        long long count;
    } profk[4];
};
