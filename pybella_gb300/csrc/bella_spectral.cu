// bella_spectral.cu -- background solve of the 3D nodal operator: the exact
// inverse of its horizontally averaged (stratified) part.
//
// The 27-point operator of lap3D (laplacian.py:898-1026) is
//   A p = (1/16) sum_d (1/dd^2) T_d H_d S_d p  (+ hcenter p),
// S_d the four-edge sum of differences along axis d on each cell, T_d the
// node sum over the four cells on either side, H_d the cell coefficient.  With
// each H_d replaced by its mean over x and z per y-cell, C_d(y), the operator
// is a sum of Kronecker products of 1D node operators: along x and z the
// difference form D^T D and the sum form M^T M, along y the tridiagonal
// D^T C D and M^T C M.  D^T D and M^T M share eigenvectors: the Hartley basis
// cas(2 pi k x / N) on a periodic axis (period N = n - 1, the duplicated seam
// averaged in and copied out) and the DCT-I basis cos(pi k i / (n - 1)) on a
// wall axis (with trapezoid weights), eigenvalues mu_k = 4 sin^2(theta_k / 2)
// and 4 - mu_k.  So the background operator is inverted by
//   forward transform in z, forward transform in x (dense FP32 GEMMs),
//   one FP64 tridiagonal solve along y per (kx, kz) mode,
//   inverse transform in x, inverse transform in z.
// Every coefficient field of this operator has the same null space (the
// kernel of S: constants and the hourglass modes f(i)(-1)^(j+k), ...), so the
// background inverse preconditions A with condition number bounded by the
// spread of H_d / C_d.  Modes whose line operator is singular (the null
// space) get the pseudo-inverse: the right-hand side loses its null component,
// one unknown is pinned, the solution loses its null component.  The hcenter
// term enters through its horizontal mean per y-node (exact on the interior);
// the Coriolis cross terms are not part of the background.  No counterpart
// in the reference, whose solve is unpreconditioned (second_projection.py:230).
#include <cmath>
#include <cstring>
#include <vector>

#include "bella_internal.cuh"

struct bella_spectral3d {
    int device;
    int nx, ny, nz;
    int xper, zper;        // 1: periodic axis (Hartley), 0: wall (DCT-I)
    int Kx, Kz;            // modes per axis
    int hc_zero;           // no hcenter term: singular mode lines exist
    long long n;
    float *txf, *txi;      // [Kx][nx], [nx][Kx]
    float *tzfT, *tziT;    // [nz][Kz], [Kz][nz] (transposed for the GEMMs)
    double *mux, *muz;     // eigenvalues of D^T D per mode
    double *cx, *cy, *cz;  // y-cell means (ny - 1 interior cells)
    double *hcm;           // y-node means of hcenter (ny)
    double *mpart;         // partial sums of the means (ny * SP_CHUNKS * 4)
    float *dscale;         // 1 / diag_inv
    float *w1, *w2;        // transform work arrays (n floats each)
    float *c1, *c2;        // work arrays of a preconditioner composed with the network
    float *la, *lc, *li;   // Thomas factors of every mode line, [ny][Kx*Kz] each
    double idx2, idy2, idz2;
    int fft_x, fft_z;      // 1: this axis transforms by FFT (power-of-two length), 0: by GEMM
    int twod;              // the 2D 9-point operator: one transformed axis (x, in the z role), no x pass
    int Lx, Lz;            // FFT lengths
    float2 *twx, *twz;     // twiddles exp(-2 pi i t / L), t < L/2
    long long launches;
};

namespace bella {

constexpr int SG_BM = 128, SG_BN = 128, SG_BK = 8, SG_THREADS = 256;

// C[M][N] = A[M][K] * B[K][N], row-major with leading dimensions; with SCALE
// every element of A is multiplied by As (same layout) as it is loaded.
// 128x128 tile per CTA, 8x8 outputs per thread (rows ty*4+i, ty*4+64+i and
// columns tx*4+j, tx*4+64+j, so shared-memory reads are conflict-free), k
// staged 8 at a time with a register prefetch of the next slab.  Threads whose
// rows or columns all lie outside the matrix skip the arithmetic.
template <bool SCALE>
__global__ void __launch_bounds__(SG_THREADS, 2)
k_sgemm(int M, int N, int K, const float *__restrict__ A, long long lda, const float *__restrict__ As,
        const float *__restrict__ B, long long ldb, float *__restrict__ C, long long ldc) {
    __shared__ __align__(16) float sa[2][SG_BK][SG_BM];
    __shared__ __align__(16) float sb[2][SG_BK][SG_BN];
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const long long m0 = (long long)blockIdx.y * SG_BM, n0 = (long long)blockIdx.x * SG_BN;
    // loader coordinates
    const int a_row = t >> 1, a_k = (t & 1) * 4;          // A: 128 rows x 8 k
    const int b_k = t >> 5, b_col = (t & 31) * 4;          // B: 8 k x 128 columns
    float ra[4], rb[4];
    auto load = [&](int k0) {
        const long long gm = m0 + a_row;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int gk = k0 + a_k + q;
            float v = 0.f;
            if (gm < M && gk < K) {
                v = A[gm * lda + gk];
                if (SCALE) v *= As[gm * lda + gk];
            }
            ra[q] = v;
        }
        const int gk = k0 + b_k;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long gn = n0 + b_col + q;
            rb[q] = (gk < K && gn < N) ? B[(long long)gk * ldb + gn] : 0.f;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 4; ++q) sa[buf][a_k + q][a_row] = ra[q];
        *reinterpret_cast<float4 *>(&sb[buf][b_k][b_col]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
    };
    const bool rows_live = (m0 + ty * 4 < M) || (m0 + ty * 4 + 64 < M);
    const bool cols_live = (n0 + tx * 4 < N) || (n0 + tx * 4 + 64 < N);
    const bool live = rows_live && cols_live;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    const int nk = (K + SG_BK - 1) / SG_BK;
    load(0);
    store(0);
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int cur = kt & 1;
        if (kt + 1 < nk) load((kt + 1) * SG_BK);
        if (live) {
#pragma unroll
            for (int kk = 0; kk < SG_BK; ++kk) {
                const float4 a0 = *reinterpret_cast<const float4 *>(&sa[cur][kk][ty * 4]);
                const float4 a1 = *reinterpret_cast<const float4 *>(&sa[cur][kk][ty * 4 + 64]);
                const float4 b0 = *reinterpret_cast<const float4 *>(&sb[cur][kk][tx * 4]);
                const float4 b1 = *reinterpret_cast<const float4 *>(&sb[cur][kk][tx * 4 + 64]);
                const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
            }
        }
        if (kt + 1 < nk) {
            store(cur ^ 1);
            __syncthreads();
        }
    }
    if (!live) return;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const long long gm = m0 + ty * 4 + (i & 3) + (i >= 4 ? 64 : 0);
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const long long gn = n0 + tx * 4 + (j & 3) + (j >= 4 ? 64 : 0);
            if (gn < N) C[gm * ldc + gn] = acc[i][j];
        }
    }
}

static void sgemm(int M, int N, int K, const float *A, long long lda, const float *As, const float *B, long long ldb,
                  float *C, long long ldc, cudaStream_t s) {
    dim3 grid((N + SG_BN - 1) / SG_BN, (M + SG_BM - 1) / SG_BM);
    if (As) k_sgemm<true><<<grid, SG_THREADS, 0, s>>>(M, N, K, A, lda, As, B, ldb, C, ldc);
    else k_sgemm<false><<<grid, SG_THREADS, 0, s>>>(M, N, K, A, lda, nullptr, B, ldb, C, ldc);
}

// ---- FFT path of the transforms (power-of-two lengths 16..2048) ---------------
// Every line of the axis is transformed by a two-pass FFT, L = R1 * R2 (R1 = 16,
// or 32 for L = 2048):
//   X[k1 + R1 k2] = sum_n2 W_R2^(n2 k2) W_L^(n2 k1) sum_n1 W_R1^(n1 k1) x[R2 n1 + n2]
// pass A: one thread per (line, n2) does the R1-point DFT in registers and the
// twiddle W_L^(n2 k1), writing through shared memory; pass B: one thread per
// (line, k1) does the R2-point DFT in registers and writes the outputs.
//   Hartley (periodic axis, N = n - 1 = L):  H_k = Re F_k - Im F_k of the FFT of
//     p (p_0 = (r_0 + r_N)/2 on the duplicated seam); inverse: the same with 1/N,
//     the seam copied out.
//   DCT-I (wall axis, M = n - 1, L = 2M):  S_k = sum_{i=0..M} cos(pi k i / M) r_i
//     = (Y_k + r_0 + (-1)^k r_M) / 2 with Y the FFT of the even extension
//     (r_0 .. r_M, r_{M-1} .. r_1); forward divides by the DCT-I norms, the
//     inverse is S itself.
// Line l of the axis has its t-th value at l * lmul + t * ts (z lines: lmul =
// row length, ts = 1; x lines: lmul = 1, ts = ny * Kz).  Threads run along t for
// z lines and across lines for x lines, so global accesses are coalesced both
// ways, and the shared-memory layout follows the same order.
constexpr int FFT_R1 = 16;
__constant__ float2 c_tw64[64];            // exp(-2 pi i t / 64)

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__host__ __device__ constexpr int bitrev_c(int i, int R) {
    int r = 0;
    for (int b = 1; b < R; b <<= 1) {
        r = (r << 1) | (i & 1);
        i >>= 1;
    }
    return r;
}

// one radix-2 stage (butterflies of span LEN) of an in-register FFT of R values,
// then the next stage; every index is a compile-time constant
template <int R, int LEN>
struct RegStage {
    static __device__ __forceinline__ void run(float2 (&v)[R]) {
#pragma unroll
        for (int i = 0; i < R; i += LEN) {
#pragma unroll
            for (int k = 0; k < LEN / 2; ++k) {
                const float2 w = c_tw64[k * (64 / LEN)];
                const float2 u = v[i + k], t = cmulf(w, v[i + k + LEN / 2]);
                v[i + k] = make_float2(u.x + t.x, u.y + t.y);
                v[i + k + LEN / 2] = make_float2(u.x - t.x, u.y - t.y);
            }
        }
        RegStage<R, 2 * LEN>::run(v);
    }
};
template <int R>
struct RegStage<R, 2 * R> {
    static __device__ __forceinline__ void run(float2 (&)[R]) {}
};

// forward DFT of R (power of two, <= 64) values in registers, natural order out
template <int R>
__device__ __forceinline__ void reg_fft(float2 (&v)[R]) {
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int j = bitrev_c(i, R);
        if (j > i) {
            const float2 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
    RegStage<R, 2>::run(v);
}
template <>
__device__ __forceinline__ void reg_fft<1>(float2 (&)[1]) {}

template <int R1, int R2>
struct FftShape {
    static constexpr int L = R1 * R2;
    // lines per CTA: pass A runs R2 threads per line; at most 6144 complex values
    // of shared memory (48 KB of static shared memory with the padding)
    static constexpr int LPC_A = (256 / R2) < 128 ? (256 / R2) : 128;
    static constexpr int LPC_S = 6144 / (R1 * (R2 + 1));
    static constexpr int LPC = LPC_A < LPC_S ? LPC_A : LPC_S;
    static constexpr int SMEM = LPC * R1 * (R2 + 1) > R1 * R2 * (LPC + 1) ? LPC * R1 * (R2 + 1)
                                                                          : R1 * R2 * (LPC + 1);
};

template <int KIND, bool FWD, int R1, int R2>   // KIND 0: Hartley, 1: DCT-I
__global__ void __launch_bounds__(256)
k_sp_fft(long long nlines, const float *__restrict__ in, long long in_lmul, long long in_ts,
         const float *__restrict__ scale, float *__restrict__ out, long long out_lmul, long long out_ts,
         const float2 *__restrict__ twL) {
    constexpr int L = FftShape<R1, R2>::L, M = L / 2, LPC = FftShape<R1, R2>::LPC;
    __shared__ float2 S[FftShape<R1, R2>::SMEM];
    const long long l0 = (long long)blockIdx.x * LPC;
    const int nl = (int)(nlines - l0 < LPC ? nlines - l0 : LPC);
    const bool ic = in_ts == 1, oc = out_ts == 1;
    // shared layout: [line][k1][n2] (padded rows) when threads run along a line,
    // [k1][n2][line] (padded) when they run across lines
    auto sidx = [&](int line, int k1, int n2) {
        return ic ? (line * R1 + k1) * (R2 + 1) + n2 : (k1 * R2 + n2) * (LPC + 1) + line;
    };
    auto ld = [&](long long g) {
        float v = in[g];
        if (scale) v *= scale[g];
        return v;
    };
    for (int q = threadIdx.x; q < nl * R2; q += blockDim.x) {
        const int line = ic ? q / R2 : q % nl, n2 = ic ? q % R2 : q / nl;
        const long long base = (l0 + line) * in_lmul;
        float2 v[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; ++n1) {
            const int j = R2 * n1 + n2;
            float x;
            if (KIND == 0)
                x = (FWD && j == 0) ? 0.5f * (ld(base) + ld(base + (long long)L * in_ts)) : ld(base + (long long)j * in_ts);
            else
                x = ld(base + (long long)(j <= M ? j : L - j) * in_ts);
            v[n1] = make_float2(x, 0.f);
        }
        reg_fft<R1>(v);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) S[sidx(line, k1, n2)] = cmulf(twL[n2 * k1], v[k1]);
    }
    __syncthreads();
    const int nout = KIND == 0 ? L : M + 1;
    for (int q = threadIdx.x; q < nl * R1; q += blockDim.x) {
        const int line = ic ? q / R1 : q % nl, k1 = ic ? q % R1 : q / nl;
        float2 u[R2];
#pragma unroll
        for (int n2 = 0; n2 < R2; ++n2) u[n2] = S[sidx(line, k1, n2)];
        reg_fft<R2>(u);
        const long long obase = (l0 + line) * out_lmul;
        float e0 = 0.f, eM = 0.f;
        if (KIND == 1) {
            const long long base = (l0 + line) * in_lmul;
            e0 = ld(base);
            eM = ld(base + (long long)M * in_ts);
        }
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            const int k = k1 + R1 * k2;
            if (k >= nout) continue;
            float val;
            if (KIND == 0) {
                val = u[k2].x - u[k2].y;
                if (!FWD) val *= 1.f / (float)L;
            } else {
                val = 0.5f * (u[k2].x + e0 + ((k & 1) ? -eM : eM));
                if (FWD) val *= (k == 0 || k == M) ? 1.f / (float)M : 2.f / (float)M;
            }
            out[obase + (long long)k * out_ts] = val;
            if (KIND == 0 && !FWD && k == 0) out[obase + (long long)L * out_ts] = val;   // seam copy
        }
    }
    (void)oc;
}

template <int KIND, bool FWD>
static void sp_fft(long long nlines, int L, const float *in, long long in_lmul, long long in_ts, const float *scale,
                   float *out, long long out_lmul, long long out_ts, const float2 *tw, cudaStream_t s) {
#define BELLA_FFT_CASE(R1, R2)                                                                                  \
    case R1 * R2: {                                                                                             \
        const unsigned grid = (unsigned)((nlines + FftShape<R1, R2>::LPC - 1) / FftShape<R1, R2>::LPC);         \
        k_sp_fft<KIND, FWD, R1, R2><<<grid, 256, 0, s>>>(nlines, in, in_lmul, in_ts, scale, out, out_lmul, out_ts, \
                                                         tw);                                                   \
        break;                                                                                                  \
    }
    switch (L) {
        BELLA_FFT_CASE(16, 1)
        BELLA_FFT_CASE(16, 2)
        BELLA_FFT_CASE(16, 4)
        BELLA_FFT_CASE(16, 8)
        BELLA_FFT_CASE(16, 16)
        BELLA_FFT_CASE(16, 32)
        BELLA_FFT_CASE(16, 64)
        BELLA_FFT_CASE(32, 64)
        default: break;
    }
#undef BELLA_FFT_CASE
}

// y-cell means of the three cell coefficients over the interior x and z cells
// (cells 1..n-1: one period on a periodic axis, the cells between walls on a
// wall axis) and y-node means of hcenter.  Block (j, c) sums chunk c of y index
// j into part[(j * SP_CHUNKS + c) * 4 + v]; k_sp_means_final adds the chunks in
// order (deterministic).
constexpr int SP_CHUNKS = 16;

__global__ void __launch_bounds__(256)
k_sp_means(int nx, int ny, int nz, const double *hx, const double *hy, const double *hz, const double *hc,
           double *part) {
    const int j = blockIdx.x, c = blockIdx.y;
    __shared__ double red[4][256];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    const long long cyz = (long long)(ny + 1) * (nz + 1);
    const long long step = (long long)blockDim.x * SP_CHUNKS;
    if (j >= 1) {                             // y-cell j (between nodes j-1 and j)
        for (long long q = (long long)c * blockDim.x + threadIdx.x; q < (long long)(nx - 1) * (nz - 1); q += step) {
            const long long i = 1 + q / (nz - 1), k = 1 + q % (nz - 1);
            const long long cc = i * cyz + (long long)j * (nz + 1) + k;
            a[0] += hx[cc];
            a[1] += hy[cc];
            a[2] += hz[cc];
        }
    }
    if (hc) {
        for (long long q = (long long)c * blockDim.x + threadIdx.x; q < (long long)nx * nz; q += step) {
            const long long i = q / nz, k = q % nz;
            a[3] += hc[(i * ny + j) * nz + k];
        }
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) red[v][threadIdx.x] = a[v];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int v = 0; v < 4; ++v) red[v][threadIdx.x] += red[v][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[((long long)j * SP_CHUNKS + c) * 4 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_sp_means_final(int nx, int ny, int nz, int has_hc, const double *part, double *cx, double *cy,
                                 double *cz, double *hcm) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ny) return;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < SP_CHUNKS; ++c)
        for (int v = 0; v < 4; ++v) a[v] += part[((long long)j * SP_CHUNKS + c) * 4 + v];
    if (j >= 1) {
        const double inv = 1.0 / ((double)(nx - 1) * (nz - 1));
        cx[j - 1] = a[0] * inv;
        cy[j - 1] = a[1] * inv;
        cz[j - 1] = a[2] * inv;
    }
    hcm[j] = has_hc ? a[3] / ((double)nx * nz) : 0.0;
}

// 2D operator (cells (ny+1) x (nx+1), row stride nx+1; nodes ny x nx): per interior
// y-cell row a = 1..ny-1, the mean over the interior columns 1..nx-1 of cxx*hplusx
// and cyy*hplusy; per node row, the mean of hcenter.  Block (a, c) sums chunk c into
// part[(a * SP_CHUNKS + c) * 4 + v] (v: 2 -> x coefficient, 1 -> y coefficient, 3 -> hcenter).
__global__ void __launch_bounds__(256)
k_sp2_means(int nx, int ny, const double *hx, const double *hy, const double *cxx, const double *cyy,
            const double *hc, double *part) {
    const int a = blockIdx.x, c = blockIdx.y;
    __shared__ double red[4][256];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 1 + c * (int)blockDim.x + (int)threadIdx.x; b <= nx - 1 && a >= 1; b += (int)blockDim.x * SP_CHUNKS) {
        const long long q = (long long)a * (nx + 1) + b;
        v[1] += cyy[q] * hy[q];
        v[2] += cxx[q] * hx[q];
    }
    if (hc && a < ny)
        for (int i = c * (int)blockDim.x + (int)threadIdx.x; i < nx; i += (int)blockDim.x * SP_CHUNKS)
            v[3] += hc[(long long)a * nx + i];
#pragma unroll
    for (int q = 0; q < 4; ++q) red[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[((long long)a * SP_CHUNKS + c) * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// the 2D means in the 3D roles: cy = mean(cyy hplusy), cz = mean(cxx hplusx), cx = 0
__global__ void k_sp2_means_final(int nx, int ny, int has_hc, const double *part, double *cx, double *cy,
                                  double *cz, double *hcm) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= ny) return;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < SP_CHUNKS; ++c)
        for (int q = 0; q < 4; ++q) v[q] += part[((long long)a * SP_CHUNKS + c) * 4 + q];
    if (a >= 1) {
        const double inv = 1.0 / (double)(nx - 1);
        cx[a - 1] = 0.0;
        cy[a - 1] = v[1] * inv;
        cz[a - 1] = v[2] * inv;
    }
    hcm[a] = has_hc ? v[3] / (double)nx : 0.0;
}

__global__ void k_sp_recip(long long n, const double *dinv, float *out) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x)
        out[g] = 1.f / (float)dinv[g];
}

// Line operator of mode (kx, kz): alpha M^T Cx M + beta D^T Cy D + gamma M^T Cz M
// + diag(hcm) with alpha = -mux (4 - muz) / (16 dx^2), beta = -(4 - mux)(4 - muz) /
// (16 dy^2), gamma = -(4 - mux) muz / (16 dz^2).  Without hcenter three kinds of
// line are singular: alpha = gamma = 0 (null vector: constants, cat 1), beta = 0
// (null vector (-1)^j, cat 2) and all zero (cat 3, output 0).
struct LineCoef {
    double al, be, ga;
    int cat;
};

__device__ __forceinline__ LineCoef line_coef(int kx, int kz, const double *mux, const double *muz, int hc_zero,
                                              double idx2, double idy2, double idz2) {
    const double mx = mux[kx], mz = muz[kz];
    LineCoef c;
    c.al = -0.0625 * mx * (4.0 - mz) * idx2;
    c.be = -0.0625 * (4.0 - mx) * (4.0 - mz) * idy2;
    c.ga = -0.0625 * (4.0 - mx) * mz * idz2;
    c.cat = 0;
    if (hc_zero) {
        if (c.al == 0.0 && c.be == 0.0 && c.ga == 0.0) c.cat = 3;
        else if (c.al == 0.0 && c.ga == 0.0) c.cat = 1;
        else if (c.be == 0.0) c.cat = 2;
    }
    return c;
}

// Thomas factors of every mode line, once per operator, computed in FP64 and
// stored in FP32: la[j] (sub-diagonal, 0 on the first solved row), lc[j] = c'_j,
// li[j] = 1 / (b_j - a_j c'_{j-1}); a singular line pins x_0 = 0 and is factored
// from row 1.  Layout [j][line].
__global__ void __launch_bounds__(128)
k_sp_factor(int Kx, int ny, int Kz, const double *mux, const double *muz, const double *cx, const double *cy,
            const double *cz, const double *hcm, int hc_zero, double idx2, double idy2, double idz2, float *la,
            float *lc, float *li) {
    const long long nl = (long long)Kx * Kz;
    const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (line >= nl) return;
    const LineCoef L = line_coef((int)(line / Kz), (int)(line % Kz), mux, muz, hc_zero, idx2, idy2, idz2);
    if (L.cat == 3) return;
    // row j couples nodes j-1, j, j+1 through the cells j-1 and j (cx, cy, cz per cell
    // row, ny-1 of them): off-diagonal al cx - be cy + ga cz of a cell, diagonal hcm plus
    // al cx + be cy + ga cz of both cells.  A row's cell coefficients and off-diagonal
    // carry over to the next row, so each row costs one new cell (12 FP64 operations
    // with the reciprocal; GB300's FP64 pipe bounds this loop)
    const int j0 = L.cat ? 1 : 0;
    double px = j0 > 0 ? cx[j0 - 1] : 0.0, py = j0 > 0 ? cy[j0 - 1] : 0.0, pz = j0 > 0 ? cz[j0 - 1] : 0.0;
    double a = 0.0, cprev = 0.0;                      // no sub-diagonal in the first solved row
    for (int j = j0; j < ny; ++j) {
        const bool last = j == ny - 1;
        const double qx = last ? 0.0 : cx[j], qy = last ? 0.0 : cy[j], qz = last ? 0.0 : cz[j];
        const double c = L.al * qx - L.be * qy + L.ga * qz;                       // 0 on the last row
        const double d = hcm[j] + L.al * (px + qx) + L.be * (py + qy) + L.ga * (pz + qz);
        // 1 / den by Newton-Raphson from an FP32 seed: each step x <- x (2 - den x)
        // squares the relative error (2^-23 -> 2^-46 -> below FP64 rounding), four
        // FP64 FMAs instead of an FP64 division
        const double den = d - a * cprev;
        double inv;
        if (fabs(den) > 1e-30 && fabs(den) < 1e30) {   // the seed within FP32's range
            inv = (double)(1.0f / (float)den);
            inv = inv * fma(-den, inv, 2.0);
            inv = inv * fma(-den, inv, 2.0);
        } else {
            inv = 1.0 / den;
        }
        cprev = c * inv;
        la[(long long)j * nl + line] = (float)a;
        lc[(long long)j * nl + line] = (float)cprev;
        li[(long long)j * nl + line] = (float)inv;
        a = c;
        px = qx; py = qy; pz = qz;
    }
}

// One Thomas solve along y per (kx, kz) mode with the precomputed factors, in
// place on W [Kx][ny][Kz] (a mode's values are Kz apart; consecutive threads
// take consecutive kz, so every access is coalesced across the warp).  The
// sweeps run in FP32 with the factors computed in FP64 (GB300's FP64 pipe runs
// at 1/64 of the FP32 rate and would bound this kernel); the null-component
// sums of the few singular lines stay in FP64.
__global__ void __launch_bounds__(128)
k_sp_lines(int Kx, int ny, int Kz, float *__restrict__ W, const double *__restrict__ mux,
           const double *__restrict__ muz, int hc_zero, double idx2, double idy2, double idz2,
           const float *__restrict__ la, const float *__restrict__ lc, const float *__restrict__ li) {
    const long long nl = (long long)Kx * Kz;
    const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (line >= nl) return;
    const int kx = (int)(line / Kz), kz = (int)(line % Kz);
    const LineCoef L = line_coef(kx, kz, mux, muz, hc_zero, idx2, idy2, idz2);
    float *__restrict__ w = W + (long long)kx * ny * Kz + kz;
    if (L.cat == 3) {
        for (int j = 0; j < ny; ++j) w[(long long)j * Kz] = 0.f;
        return;
    }
    float proj = 0.f;
    if (L.cat) {                               // remove the right-hand side's null component
        double ps = 0.0;
        for (int j = 0; j < ny; ++j) ps += (L.cat == 2 && (j & 1)) ? -(double)w[(long long)j * Kz] : (double)w[(long long)j * Kz];
        proj = (float)(ps / ny);
    }
    // sweeps in batches of 12 rows: the loads of a batch are issued before its
    // dependent arithmetic, and its stores after it (the in-place rows would
    // otherwise serialise every load behind the previous row's store)
    constexpr int B = 12;
    const int j0 = L.cat ? 1 : 0;
    float d = 0.f;
    for (int jb = j0; jb < ny; jb += B) {
        float r[B], a[B], iv[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int j = jb + u;
            if (j < ny) {
                const long long q = (long long)j * nl + line;
                r[u] = w[(long long)j * Kz];
                a[u] = la[q];
                iv[u] = li[q];
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int j = jb + u;
            if (j < ny) {
                float rhs = r[u];
                if (L.cat) rhs -= (L.cat == 2 && (j & 1)) ? -proj : proj;
                d = fmaf(-a[u], d, rhs) * iv[u];
                r[u] = d;
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (jb + u < ny) w[(long long)(jb + u) * Kz] = r[u];
    }
    float x = 0.f;
    double sum = 0.0;
    for (int jt = ny - 1; jt >= j0; jt -= B) {
        float r[B], c[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int j = jt - u;
            if (j >= j0) {
                r[u] = w[(long long)j * Kz];
                c[u] = lc[(long long)j * nl + line];
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int j = jt - u;
            if (j >= j0) {
                x = fmaf(-c[u], x, r[u]);
                r[u] = x;
                if (L.cat) sum += (L.cat == 2 && (j & 1)) ? -(double)x : (double)x;
            }
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (jt - u >= j0) w[(long long)(jt - u) * Kz] = r[u];
    }
    if (!L.cat) return;
    const float shift = (float)(sum / ny);     // x_0 = 0 pinned; remove the null component
    w[0] = -shift;
    for (int j = j0; j < ny; ++j) w[(long long)j * Kz] -= (L.cat == 2 && (j & 1)) ? -shift : shift;
}

// out = A_bg^+ (in / diag_inv): the background inverse applied to a residual of
// the Jacobi-scaled system; FP32 in and out.
int spectral_apply_dev(bella_spectral3d *sp, const float *in, float *out, cudaStream_t s) {
    const int nx = sp->nx, ny = sp->ny, nz = sp->nz, Kx = sp->Kx, Kz = sp->Kz;
    const long long rows = (long long)nx * ny, xl = (long long)ny * Kz;
    if (sp->twod) {                                       // one transformed axis: rows of nz values
        const long long nl = Kz;
        if (sp->fft_z) {
            if (sp->zper) sp_fft<0, true>(rows, sp->Lz, in, nz, 1, sp->dscale, sp->w2, Kz, 1, sp->twz, s);
            else sp_fft<1, true>(rows, sp->Lz, in, nz, 1, sp->dscale, sp->w2, Kz, 1, sp->twz, s);
        } else {
            sgemm(ny, Kz, nz, in, nz, sp->dscale, sp->tzfT, Kz, sp->w2, Kz, s);
        }
        k_sp_lines<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(1, ny, Kz, sp->w2, sp->mux, sp->muz, sp->hc_zero,
                                                                sp->idx2, sp->idy2, sp->idz2, sp->la, sp->lc,
                                                                sp->li);
        if (sp->fft_z) {
            if (sp->zper) sp_fft<0, false>(rows, sp->Lz, sp->w2, Kz, 1, nullptr, out, nz, 1, sp->twz, s);
            else sp_fft<1, false>(rows, sp->Lz, sp->w2, Kz, 1, nullptr, out, nz, 1, sp->twz, s);
        } else {
            sgemm(ny, nz, Kz, sp->w2, Kz, nullptr, sp->tziT, nz, out, nz, s);
        }
        sp->launches += 3;
        return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
    }
    // z forward: w1[(x,y)][kz] from in[(x,y)][z] / dinv
    if (sp->fft_z) {
        if (sp->zper) sp_fft<0, true>(rows, sp->Lz, in, nz, 1, sp->dscale, sp->w1, Kz, 1, sp->twz, s);
        else sp_fft<1, true>(rows, sp->Lz, in, nz, 1, sp->dscale, sp->w1, Kz, 1, sp->twz, s);
    } else {
        sgemm(nx * ny, Kz, nz, in, nz, sp->dscale, sp->tzfT, Kz, sp->w1, Kz, s);
    }
    // x forward: w2[kx][(y,kz)] from w1[x][(y,kz)]
    if (sp->fft_x) {
        if (sp->xper) sp_fft<0, true>(xl, sp->Lx, sp->w1, 1, xl, nullptr, sp->w2, 1, xl, sp->twx, s);
        else sp_fft<1, true>(xl, sp->Lx, sp->w1, 1, xl, nullptr, sp->w2, 1, xl, sp->twx, s);
    } else {
        sgemm(Kx, ny * Kz, nx, sp->txf, nx, nullptr, sp->w1, xl, sp->w2, xl, s);
    }
    const long long nl = (long long)Kx * Kz;
    k_sp_lines<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(Kx, ny, Kz, sp->w2, sp->mux, sp->muz, sp->hc_zero,
                                                            sp->idx2, sp->idy2, sp->idz2, sp->la, sp->lc, sp->li);
    // x inverse: w1[x][(y,kz)] from w2[kx][(y,kz)]
    if (sp->fft_x) {
        if (sp->xper) sp_fft<0, false>(xl, sp->Lx, sp->w2, 1, xl, nullptr, sp->w1, 1, xl, sp->twx, s);
        else sp_fft<1, false>(xl, sp->Lx, sp->w2, 1, xl, nullptr, sp->w1, 1, xl, sp->twx, s);
    } else {
        sgemm(nx, ny * Kz, Kx, sp->txi, Kx, nullptr, sp->w2, xl, sp->w1, xl, s);
    }
    // z inverse: out[(x,y)][z] from w1[(x,y)][kz]
    if (sp->fft_z) {
        if (sp->zper) sp_fft<0, false>(rows, sp->Lz, sp->w1, Kz, 1, nullptr, out, nz, 1, sp->twz, s);
        else sp_fft<1, false>(rows, sp->Lz, sp->w1, Kz, 1, nullptr, out, nz, 1, sp->twz, s);
    } else {
        sgemm(nx * ny, nz, Kz, sp->w1, Kz, nullptr, sp->tziT, nz, out, nz, s);
    }
    sp->launches += 5;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

float *spectral_work(bella_spectral3d *sp, int which) { return which ? sp->c2 : sp->c1; }
long long spectral_size(const bella_spectral3d *sp) { return sp->n; }

// eigenvalues of D^T D and (dense = 1, the GEMM path) the forward / inverse
// transform matrices of one axis
static void axis_basis(int n, int periodic, int dense, std::vector<double> &mu, std::vector<float> &fwd,
                       std::vector<float> &inv, int &K) {
    const double pi = 3.14159265358979323846;
    if (periodic) {
        const int N = n - 1;
        K = N;
        mu.assign(K, 0.0);
        for (int k = 0; k < K; ++k) {
            const double sk = sin(pi * k / N);
            mu[k] = 4.0 * sk * sk;
        }
        mu[0] = 0.0;
        if (N % 2 == 0) mu[N / 2] = 4.0;
        if (!dense) return;
        fwd.assign((size_t)K * n, 0.f);
        inv.assign((size_t)n * K, 0.f);
        for (int k = 0; k < K; ++k)
            for (int x = 0; x < n; ++x) {
                const long long kxm = ((long long)k * (x % N)) % N;    // exact phase index
                const double th = 2.0 * pi * (double)kxm / N;
                const double cas = cos(th) + sin(th);
                const double wgt = (x == 0 || x == n - 1) ? 0.5 : 1.0;
                fwd[(size_t)k * n + x] = (float)(wgt * cas);
                inv[(size_t)x * K + k] = (float)(cas / N);
            }
    } else {
        const int M = n - 1;
        K = n;
        mu.assign(K, 0.0);
        for (int k = 0; k < K; ++k) {
            const double sk = sin(0.5 * pi * k / M);
            mu[k] = 4.0 * sk * sk;
        }
        mu[0] = 0.0;
        mu[K - 1] = 4.0;
        if (!dense) return;
        fwd.assign((size_t)K * n, 0.f);
        inv.assign((size_t)n * K, 0.f);
        for (int k = 0; k < K; ++k) {
            const double nrm = (k == 0 || k == K - 1) ? (double)M : 0.5 * M;
            for (int i = 0; i < n; ++i) {
                const long long kim = ((long long)k * i) % (2 * M);
                const double c = cos(pi * (double)kim / M);
                fwd[(size_t)k * n + i] = (float)(c / nrm);
                inv[(size_t)i * K + k] = (float)c;
            }
        }
    }
}

}  // namespace bella

using namespace bella;

extern "C" {

int bella_spectral3d_destroy(bella_spectral3d *sp) {
    if (!sp) return BELLA_OK;
    cudaSetDevice(sp->device);
    void *ptrs[] = {sp->txf, sp->txi, sp->tzfT, sp->tziT, sp->mux, sp->muz, sp->cx, sp->cy, sp->cz,
                    sp->hcm, sp->mpart, sp->dscale, sp->w1, sp->w2, sp->c1, sp->c2, sp->la, sp->lc, sp->li,
                    sp->twx, sp->twz};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete sp;
    return BELLA_OK;
}

}  // extern "C"

// the parts of the set-up shared by the 3D and 2D operators: transform bases,
// allocations, means (launch_means), 1/diag_inv, Thomas factors
struct SpGeom {
    int nx, ny, nz, xper, zper, twod;
    double idx2, idy2, idz2;
    const double *dinv;
};

// the parts that depend on the operator's coefficients: y-line means, 1/diag_inv,
// the singular-line flag and the Thomas factors of every mode line.  Stream-ordered;
// it waits for the device only when the operator has an hcenter term (whose means
// decide whether singular mode lines exist).
template <typename F>
static int sp_refresh(bella_spectral3d *sp, const SpGeom &g, cudaStream_t s, F launch_means, int has_hc) {
    sp->idx2 = g.idx2;
    sp->idy2 = g.idy2;
    sp->idz2 = g.idz2;
    launch_means(sp);
    k_sp_recip<<<vec_grid(sp->n), VEC_BLOCK, 0, s>>>(sp->n, g.dinv, sp->dscale);
    sp->hc_zero = 1;
    if (has_hc) {
        std::vector<double> hcm(sp->ny);
        if (cudaMemcpyAsync(hcm.data(), sp->hcm, sp->ny * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return BELLA_ECUDA;
        for (int j = 0; j < sp->ny; ++j)
            if (hcm[j] != 0.0) sp->hc_zero = 0;
    }
    const long long nl = (long long)sp->Kx * sp->Kz;
    k_sp_factor<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(sp->Kx, sp->ny, sp->Kz, sp->mux, sp->muz, sp->cx, sp->cy,
                                                             sp->cz, sp->hcm, sp->hc_zero, sp->idx2, sp->idy2,
                                                             sp->idz2, sp->la, sp->lc, sp->li);
    sp->launches += 3;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

template <typename F>
static int sp_build(bella_spectral3d **out, const SpGeom &g, int device, cudaStream_t s, F launch_means,
                    int has_hc) {
    bella_spectral3d *sp = new bella_spectral3d;
    memset(sp, 0, sizeof(*sp));
    sp->device = device;
    sp->nx = g.nx; sp->ny = g.ny; sp->nz = g.nz;
    sp->xper = g.xper;
    sp->zper = g.zper;
    sp->twod = g.twod;
    sp->n = (long long)g.nx * g.ny * g.nz;
    sp->idx2 = g.idx2;
    sp->idy2 = g.idy2;
    sp->idz2 = g.idz2;
    // FFT path per axis when the transform length is a power of two that fits a CTA
    auto fft_len = [](int n, int periodic, int *L) {
        const int len = periodic ? n - 1 : 2 * (n - 1);
        if (len < FFT_R1 || len > 2048 || (len & (len - 1))) return 0;
        *L = len;
        return 1;
    };
    sp->fft_x = g.twod ? 0 : fft_len(g.nx, sp->xper, &sp->Lx);
    sp->fft_z = fft_len(g.nz, sp->zper, &sp->Lz);
    std::vector<double> mux, muz;
    std::vector<float> fx, ix, fz, iz;
    if (g.twod) {                         // no x axis: one mode with eigenvalue 0
        sp->Kx = 1;
        mux.assign(1, 0.0);
    } else {
        axis_basis(g.nx, sp->xper, !sp->fft_x, mux, fx, ix, sp->Kx);
    }
    axis_basis(g.nz, sp->zper, !sp->fft_z, muz, fz, iz, sp->Kz);
    const int ny = g.ny, nz = g.nz, Kx = sp->Kx, Kz = sp->Kz;
    std::vector<float> fzT, izT;
    if (!sp->fft_z) {
        fzT.resize((size_t)nz * Kz);
        izT.resize((size_t)Kz * nz);
        for (int k = 0; k < Kz; ++k)
            for (int z = 0; z < nz; ++z) {
                fzT[(size_t)z * Kz + k] = fz[(size_t)k * nz + z];
                izT[(size_t)k * nz + z] = iz[(size_t)z * Kz + k];
            }
    }
    const long long nl = (long long)Kx * Kz;
    auto upload = [&](float **dst, const std::vector<float> &v) {
        if (v.empty()) return true;
        return cudaMalloc(dst, v.size() * sizeof(float)) == cudaSuccess &&
               cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice, s) == cudaSuccess;
    };
    bool ok = upload(&sp->txf, fx) && upload(&sp->txi, ix) && upload(&sp->tzfT, fzT) && upload(&sp->tziT, izT) &&
              cudaMalloc(&sp->mux, Kx * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->muz, Kz * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cx, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cy, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cz, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->hcm, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->mpart, (size_t)ny * SP_CHUNKS * 4 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->dscale, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->w1, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->w2, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->c1, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->c2, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->la, (size_t)ny * nl * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->lc, (size_t)ny * nl * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->li, (size_t)ny * nl * sizeof(float)) == cudaSuccess;
    if (!ok) {
        bella_spectral3d_destroy(sp);
        return BELLA_ECUDA;
    }
    cudaMemcpyAsync(sp->mux, mux.data(), Kx * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->muz, muz.data(), Kz * sizeof(double), cudaMemcpyHostToDevice, s);
    auto twiddles = [&](int L, float2 **dst) {
        std::vector<float2> t(L);
        const double pi = 3.14159265358979323846;
        for (int k = 0; k < L; ++k)
            t[k] = make_float2((float)cos(2.0 * pi * k / L), (float)-sin(2.0 * pi * k / L));
        if (cudaMalloc(dst, t.size() * sizeof(float2)) != cudaSuccess) return false;
        return cudaMemcpy(*dst, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
    };
    {
        float2 t64[64];
        for (int k = 0; k < 64; ++k)
            t64[k] = make_float2((float)cos(2.0 * 3.14159265358979323846 * k / 64),
                                 (float)-sin(2.0 * 3.14159265358979323846 * k / 64));
        if (cudaMemcpyToSymbol(c_tw64, t64, sizeof(t64)) != cudaSuccess) {
            bella_spectral3d_destroy(sp);
            return BELLA_ECUDA;
        }
    }
    if ((sp->fft_x && !twiddles(sp->Lx, &sp->twx)) || (sp->fft_z && !twiddles(sp->Lz, &sp->twz))) {
        bella_spectral3d_destroy(sp);
        return BELLA_ECUDA;
    }
    if (sp_refresh(sp, g, s, launch_means, has_hc) != BELLA_OK ||
        cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        bella_spectral3d_destroy(sp);
        return BELLA_ECUDA;
    }
    *out = sp;
    return BELLA_OK;
}

// launchers of the y-line means of a 3D or 2D operator's coefficients
static auto means3d(const bella_op3d *op, cudaStream_t s) {
    return [op, s](bella_spectral3d *sp) {
        k_sp_means<<<dim3(op->ny, SP_CHUNKS), 256, 0, s>>>(op->nx, op->ny, op->nz, op->hplusx, op->hplusy, op->hplusz,
                                                           op->hcenter, sp->mpart);
        k_sp_means_final<<<(op->ny + 127) / 128, 128, 0, s>>>(op->nx, op->ny, op->nz, op->hcenter ? 1 : 0, sp->mpart,
                                                              sp->cx, sp->cy, sp->cz, sp->hcm);
    };
}
static auto means2d(const bella_op2d *op, cudaStream_t s) {
    return [op, s](bella_spectral3d *sp) {
        k_sp2_means<<<dim3(op->ny, SP_CHUNKS), 256, 0, s>>>(op->nx, op->ny, op->hplusx, op->hplusy, op->cxx, op->cyy,
                                                            op->hcenter, sp->mpart);
        k_sp2_means_final<<<(op->ny + 127) / 128, 128, 0, s>>>(op->nx, op->ny, op->hcenter ? 1 : 0, sp->mpart, sp->cx,
                                                               sp->cy, sp->cz, sp->hcm);
    };
}

extern "C" {

int bella_spectral3d_create(bella_spectral3d **out, const bella_op3d *op, int device, void *stream) {
    if (!out || !op) return BELLA_EINVAL;
    *out = nullptr;
    if (op->nx < 3 || op->ny < 3 || op->nz < 3 || !op->hplusx || !op->hplusy || !op->hplusz || !op->diag_inv)
        return BELLA_EINVAL;
    if (!op->y_wall) return BELLA_EINVAL;     // the line solves run along a walled y axis
    if (!(op->dx > 0.0) || !(op->dy > 0.0) || !(op->dz > 0.0)) return BELLA_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return BELLA_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const SpGeom g{op->nx, op->ny, op->nz, op->x_wall ? 0 : 1, op->z_wall ? 0 : 1, 0,
                   1.0 / (op->dx * op->dx), 1.0 / (op->dy * op->dy), 1.0 / (op->dz * op->dz), op->diag_inv};
    return sp_build(out, g, device, s, means3d(op, s), op->hcenter ? 1 : 0);
}

int bella_spectral3d_update(bella_spectral3d *sp, const bella_op3d *op, void *stream) {
    if (!sp || !op) return BELLA_EINVAL;
    if (sp->twod || op->nx != sp->nx || op->ny != sp->ny || op->nz != sp->nz || (op->x_wall ? 0 : 1) != sp->xper ||
        (op->z_wall ? 0 : 1) != sp->zper || !op->y_wall || !op->hplusx || !op->hplusy || !op->hplusz ||
        !op->diag_inv || !(op->dx > 0.0) || !(op->dy > 0.0) || !(op->dz > 0.0))
        return BELLA_EINVAL;
    if (cudaSetDevice(sp->device) != cudaSuccess) return BELLA_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const SpGeom g{op->nx, op->ny, op->nz, sp->xper, sp->zper, 0,
                   1.0 / (op->dx * op->dx), 1.0 / (op->dy * op->dy), 1.0 / (op->dz * op->dz), op->diag_inv};
    return sp_refresh(sp, g, s, means3d(op, s), op->hcenter ? 1 : 0);
}

int bella_spectral2d_create(bella_spectral3d **out, const bella_op2d *op, int device, void *stream) {
    if (!out || !op) return BELLA_EINVAL;
    *out = nullptr;
    if (op->nx < 3 || op->ny < 3 || !op->hplusx || !op->hplusy || !op->cxx || !op->cyy || !op->diag_inv)
        return BELLA_EINVAL;
    if (op->y_wall != 1) return BELLA_EINVAL;   // the line solves run along a walled y axis (no mirror)
    if (!(op->dx > 0.0) || !(op->dy > 0.0)) return BELLA_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return BELLA_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    // nodes [ny][nx] as the 3D layout [1][ny][nx]: x takes the role of z
    const SpGeom g{1, op->ny, op->nx, 1, op->x_wall ? 0 : 1, 1, 0.0, 1.0 / (op->dy * op->dy),
                   1.0 / (op->dx * op->dx), op->diag_inv};
    return sp_build(out, g, device, s, means2d(op, s), op->hcenter ? 1 : 0);
}

int bella_spectral2d_update(bella_spectral3d *sp, const bella_op2d *op, void *stream) {
    if (!sp || !op) return BELLA_EINVAL;
    if (!sp->twod || op->nx != sp->nz || op->ny != sp->ny || (op->x_wall ? 0 : 1) != sp->zper || op->y_wall != 1 ||
        !op->hplusx || !op->hplusy || !op->cxx || !op->cyy || !op->diag_inv || !(op->dx > 0.0) || !(op->dy > 0.0))
        return BELLA_EINVAL;
    if (cudaSetDevice(sp->device) != cudaSuccess) return BELLA_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const SpGeom g{1, op->ny, op->nx, 1, sp->zper, 1, 0.0, 1.0 / (op->dy * op->dy), 1.0 / (op->dx * op->dx),
                   op->diag_inv};
    return sp_refresh(sp, g, s, means2d(op, s), op->hcenter ? 1 : 0);
}

int bella_spectral3d_apply(bella_spectral3d *sp, const float *in, float *out, void *stream) {
    if (!sp || !in || !out) return BELLA_EINVAL;
    if (cudaSetDevice(sp->device) != cudaSuccess) return BELLA_ECUDA;
    return spectral_apply_dev(sp, in, out, (cudaStream_t)stream);
}

long long bella_spectral3d_launches(const bella_spectral3d *sp) { return sp ? sp->launches : 0; }

}  // extern "C"
