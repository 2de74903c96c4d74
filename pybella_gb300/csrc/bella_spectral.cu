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
    float *dscale;         // 1 / diag_inv
    float *w1, *w2;        // transform work arrays (n floats each)
    float *c1, *c2;        // work arrays of a preconditioner composed with the network
    double *lc, *ld;       // Thomas scratch, [ny][Kx*Kz] each
    double idx2, idy2, idz2;
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

// y-cell means of the three cell coefficients over the interior x and z cells
// (cells 1..n-1: one period on a periodic axis, the cells between walls on a
// wall axis) and y-node means of hcenter; one CTA per y index, fixed-order sums.
__global__ void __launch_bounds__(256)
k_sp_means(int nx, int ny, int nz, const double *hx, const double *hy, const double *hz, const double *hc,
           double *cx, double *cy, double *cz, double *hcm) {
    const int j = blockIdx.x;                 // 0..ny-1
    __shared__ double red[4][256];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    const long long cyz = (long long)(ny + 1) * (nz + 1);
    if (j >= 1) {                             // y-cell j (between nodes j-1 and j)
        for (long long q = threadIdx.x; q < (long long)(nx - 1) * (nz - 1); q += blockDim.x) {
            const long long i = 1 + q / (nz - 1), k = 1 + q % (nz - 1);
            const long long c = i * cyz + (long long)j * (nz + 1) + k;
            a[0] += hx[c];
            a[1] += hy[c];
            a[2] += hz[c];
        }
    }
    if (hc) {
        for (long long q = threadIdx.x; q < (long long)nx * nz; q += blockDim.x) {
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
    if (threadIdx.x == 0) {
        if (j >= 1) {
            const double inv = 1.0 / ((double)(nx - 1) * (nz - 1));
            cx[j - 1] = red[0][0] * inv;
            cy[j - 1] = red[1][0] * inv;
            cz[j - 1] = red[2][0] * inv;
        }
        hcm[j] = hc ? red[3][0] / ((double)nx * nz) : 0.0;
    }
}

__global__ void k_sp_recip(long long n, const double *dinv, float *out) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x)
        out[g] = (float)(1.0 / dinv[g]);
}

// One FP64 Thomas solve along y per (kx, kz) mode, in place on W [Kx][ny][Kz].
// Line operator: alpha M^T Cx M + beta D^T Cy D + gamma M^T Cz M + diag(hcm)
// with alpha = -mux (4 - muz) / (16 dx^2), beta = -(4 - mux)(4 - muz) / (16 dy^2),
// gamma = -(4 - mux) muz / (16 dz^2).  Without hcenter, three kinds of line are
// singular: alpha = gamma = 0 (null vector: constants), beta = 0 (null vector
// (-1)^j) and all zero (output 0).
__global__ void __launch_bounds__(128)
k_sp_lines(int Kx, int ny, int Kz, float *W, const double *mux, const double *muz, const double *cx,
           const double *cy, const double *cz, const double *hcm, int hc_zero, double idx2, double idy2, double idz2,
           double *lc, double *ld) {
    const long long nl = (long long)Kx * Kz;
    const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (line >= nl) return;
    const int kx = (int)(line / Kz), kz = (int)(line % Kz);
    const double mx = mux[kx], mz = muz[kz];
    const double al = -0.0625 * mx * (4.0 - mz) * idx2;
    const double be = -0.0625 * (4.0 - mx) * (4.0 - mz) * idy2;
    const double ga = -0.0625 * (4.0 - mx) * mz * idz2;
    float *w = W + (long long)kx * ny * Kz + kz;
    int cat = 0;
    if (hc_zero) {
        if (al == 0.0 && be == 0.0 && ga == 0.0) cat = 3;
        else if (al == 0.0 && ga == 0.0) cat = 1;
        else if (be == 0.0) cat = 2;
    }
    if (cat == 3) {
        for (int j = 0; j < ny; ++j) w[(long long)j * Kz] = 0.f;
        return;
    }
    double proj = 0.0;
    if (cat) {
        for (int j = 0; j < ny; ++j) proj += (cat == 2 && (j & 1)) ? -(double)w[(long long)j * Kz] : (double)w[(long long)j * Kz];
        proj /= ny;
    }
    auto off = [&](int j) { return al * cx[j] - be * cy[j] + ga * cz[j]; };   // between nodes j and j+1
    auto diag = [&](int j) {
        double d = hcm[j];
        if (j > 0) d += al * cx[j - 1] + be * cy[j - 1] + ga * cz[j - 1];
        if (j < ny - 1) d += al * cx[j] + be * cy[j] + ga * cz[j];
        return d;
    };
    const int j0 = cat ? 1 : 0;
    double cprev = 0.0, dprev = 0.0;
    for (int j = j0; j < ny; ++j) {
        double rhs = w[(long long)j * Kz];
        if (cat) rhs -= (cat == 2 && (j & 1)) ? -proj : proj;
        const double a = j > j0 ? off(j - 1) : 0.0;
        const double c = j < ny - 1 ? off(j) : 0.0;
        const double den = diag(j) - a * cprev;
        cprev = c / den;
        dprev = (rhs - a * dprev) / den;
        lc[(long long)j * nl + line] = cprev;
        ld[(long long)j * nl + line] = dprev;
    }
    double x = 0.0, sum = 0.0;
    for (int j = ny - 1; j >= j0; --j) {
        x = ld[(long long)j * nl + line] - (j < ny - 1 ? lc[(long long)j * nl + line] * x : 0.0);
        ld[(long long)j * nl + line] = x;
        sum += (cat == 2 && (j & 1)) ? -x : x;
    }
    const double shift = cat ? sum / ny : 0.0;   // x_0 = 0 pinned; remove the null component
    if (cat) w[0] = (float)(-shift);
    for (int j = j0; j < ny; ++j) {
        const double u = (cat == 2 && (j & 1)) ? -1.0 : 1.0;
        w[(long long)j * Kz] = (float)(ld[(long long)j * nl + line] - shift * u);
    }
}

// out = A_bg^+ (in / diag_inv): the background inverse applied to a residual of
// the Jacobi-scaled system; FP32 in and out.
int spectral_apply_dev(bella_spectral3d *sp, const float *in, float *out, cudaStream_t s) {
    const int nx = sp->nx, ny = sp->ny, nz = sp->nz, Kx = sp->Kx, Kz = sp->Kz;
    // z forward: w1[(x,y)][kz] = sum_z in[(x,y)][z] / dinv * Fz[kz][z]
    sgemm(nx * ny, Kz, nz, in, nz, sp->dscale, sp->tzfT, Kz, sp->w1, Kz, s);
    // x forward: w2[kx][(y,kz)] = sum_x Fx[kx][x] w1[x][(y,kz)]
    sgemm(Kx, ny * Kz, nx, sp->txf, nx, nullptr, sp->w1, (long long)ny * Kz, sp->w2, (long long)ny * Kz, s);
    const long long nl = (long long)Kx * Kz;
    k_sp_lines<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(Kx, ny, Kz, sp->w2, sp->mux, sp->muz, sp->cx, sp->cy,
                                                            sp->cz, sp->hcm, sp->hc_zero, sp->idx2, sp->idy2,
                                                            sp->idz2, sp->lc, sp->ld);
    // x inverse: w1[x][(y,kz)] = sum_kx Ix[x][kx] w2[kx][(y,kz)]
    sgemm(nx, ny * Kz, Kx, sp->txi, Kx, nullptr, sp->w2, (long long)ny * Kz, sp->w1, (long long)ny * Kz, s);
    // z inverse: out[(x,y)][z] = sum_kz w1[(x,y)][kz] Iz[z][kz]
    sgemm(nx * ny, nz, Kz, sp->w1, Kz, nullptr, sp->tziT, nz, out, nz, s);
    sp->launches += 5;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

float *spectral_work(bella_spectral3d *sp, int which) { return which ? sp->c2 : sp->c1; }
long long spectral_size(const bella_spectral3d *sp) { return sp->n; }

// eigenvalues of D^T D and the forward / inverse transform matrices of one axis
static void axis_basis(int n, int periodic, std::vector<double> &mu, std::vector<float> &fwd,
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
                    sp->hcm, sp->dscale, sp->w1, sp->w2, sp->c1, sp->c2, sp->lc, sp->ld};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete sp;
    return BELLA_OK;
}

int bella_spectral3d_create(bella_spectral3d **out, const bella_op3d *op, int device, void *stream) {
    if (!out || !op) return BELLA_EINVAL;
    *out = nullptr;
    if (op->nx < 3 || op->ny < 3 || op->nz < 3 || !op->hplusx || !op->hplusy || !op->hplusz || !op->diag_inv)
        return BELLA_EINVAL;
    if (!op->y_wall) return BELLA_EINVAL;     // the line solves run along a walled y axis
    if (!(op->dx > 0.0) || !(op->dy > 0.0) || !(op->dz > 0.0)) return BELLA_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return BELLA_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    bella_spectral3d *sp = new bella_spectral3d;
    memset(sp, 0, sizeof(*sp));
    sp->device = device;
    sp->nx = op->nx; sp->ny = op->ny; sp->nz = op->nz;
    sp->xper = op->x_wall ? 0 : 1;
    sp->zper = op->z_wall ? 0 : 1;
    sp->n = (long long)op->nx * op->ny * op->nz;
    sp->idx2 = 1.0 / (op->dx * op->dx);
    sp->idy2 = 1.0 / (op->dy * op->dy);
    sp->idz2 = 1.0 / (op->dz * op->dz);
    std::vector<double> mux, muz;
    std::vector<float> fx, ix, fz, iz;
    axis_basis(op->nx, sp->xper, mux, fx, ix, sp->Kx);
    axis_basis(op->nz, sp->zper, muz, fz, iz, sp->Kz);
    const int nx = op->nx, ny = op->ny, nz = op->nz, Kx = sp->Kx, Kz = sp->Kz;
    std::vector<float> fzT((size_t)nz * Kz), izT((size_t)Kz * nz);
    for (int k = 0; k < Kz; ++k)
        for (int z = 0; z < nz; ++z) {
            fzT[(size_t)z * Kz + k] = fz[(size_t)k * nz + z];
            izT[(size_t)k * nz + z] = iz[(size_t)z * Kz + k];
        }
    const long long nl = (long long)Kx * Kz;
    bool ok = cudaMalloc(&sp->txf, fx.size() * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->txi, ix.size() * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->tzfT, fzT.size() * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->tziT, izT.size() * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->mux, Kx * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->muz, Kz * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cx, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cy, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->cz, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->hcm, ny * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->dscale, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->w1, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->w2, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->c1, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->c2, sp->n * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&sp->lc, (size_t)ny * nl * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&sp->ld, (size_t)ny * nl * sizeof(double)) == cudaSuccess;
    if (!ok) {
        bella_spectral3d_destroy(sp);
        return BELLA_ECUDA;
    }
    cudaMemcpyAsync(sp->txf, fx.data(), fx.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->txi, ix.data(), ix.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->tzfT, fzT.data(), fzT.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->tziT, izT.data(), izT.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->mux, mux.data(), Kx * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(sp->muz, muz.data(), Kz * sizeof(double), cudaMemcpyHostToDevice, s);
    k_sp_means<<<ny, 256, 0, s>>>(nx, ny, nz, op->hplusx, op->hplusy, op->hplusz, op->hcenter, sp->cx, sp->cy,
                                  sp->cz, sp->hcm);
    k_sp_recip<<<vec_grid(sp->n), VEC_BLOCK, 0, s>>>(sp->n, op->diag_inv, sp->dscale);
    std::vector<double> hcm(ny);
    cudaMemcpyAsync(hcm.data(), sp->hcm, ny * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        bella_spectral3d_destroy(sp);
        return BELLA_ECUDA;
    }
    sp->hc_zero = 1;
    for (int j = 0; j < ny; ++j)
        if (hcm[j] != 0.0) sp->hc_zero = 0;
    sp->launches = 2;
    *out = sp;
    return BELLA_OK;
}

int bella_spectral3d_apply(bella_spectral3d *sp, const float *in, float *out, void *stream) {
    if (!sp || !in || !out) return BELLA_EINVAL;
    if (cudaSetDevice(sp->device) != cudaSuccess) return BELLA_ECUDA;
    return spectral_apply_dev(sp, in, out, (cudaStream_t)stream);
}

long long bella_spectral3d_launches(const bella_spectral3d *sp) { return sp ? sp->launches : 0; }

}  // extern "C"
