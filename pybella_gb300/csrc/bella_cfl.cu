// bella_cfl.cu -- the maxima of the reference's CFL time step (cfl.py:5-74) over
// the device state: |u|, |v|, |w| and |u|+c, |v|+c, |w|+c with the sound speed
// c = sqrt(gamma rhoY^gamma / rho) / sqrt(Msq), over every cell (ghosts included,
// as the reference takes .max() of the whole arrays).  One thread per cell, a
// block maximum, then an atomic maximum on the bit patterns (non-negative doubles
// order as their bit patterns do).  The time step itself is host arithmetic.
// A NaN anywhere (a blown-up state, or rhoY < 0 under pow) makes that maximum NaN,
// as numpy's .max() does: the maxima propagate NaN (fmax would drop it), and a NaN's
// bit pattern, either sign, is above +inf's as an unsigned integer, so the atomic
// maximum keeps it.
#include <cstring>

#include "bella_internal.cuh"

namespace bella {

// maximum that keeps a NaN of either operand
__device__ __forceinline__ double nan_max(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }

__global__ void k_cfl_maxima(long long n, const double *rho, const double *rhou, const double *rhov,
                             const double *rhow, const double *rhoY, double gamm, double Minv,
                             unsigned long long *out) {
    __shared__ double red[6][8];
    double m[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double p = pow(rhoY[e], gamm);
        const double c = sqrt(gamm * p / rho[e]) * Minv;
        const double u = fabs(rhou[e] / rho[e]), v = fabs(rhov[e] / rho[e]), w = fabs(rhow[e] / rho[e]);
        const double q[6] = {u, v, w, u + c, v + c, w + c};
        for (int k = 0; k < 6; ++k) m[k] = nan_max(m[k], q[k]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 6; ++k) {
        double v = m[k];
        for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = nan_max(v, red[threadIdx.x][w]);
        atomicMax(&out[threadIdx.x], (unsigned long long)__double_as_longlong(v));
    }
}

}  // namespace bella

using namespace bella;

extern "C" int bella_cfl_maxima(const double *rho, const double *rhou, const double *rhov, const double *rhow,
                                const double *rhoY, long long n, double gamm, double Msq, void *scratch,
                                double *out, void *stream) {
    if (!rho || !rhou || !rhov || !rhow || !rhoY || !out || !scratch)
        return set_err(BELLA_EINVAL, "bella_cfl_maxima: null pointer");
    if (n <= 0 || !(Msq > 0.0)) return set_err(BELLA_EINVAL, "bella_cfl_maxima: n <= 0 or Msq <= 0");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *d = (unsigned long long *)scratch;
    int rc = cuda_check(cudaMemsetAsync(d, 0, 6 * sizeof(unsigned long long), s), "bella_cfl_maxima: memset");
    if (rc != BELLA_OK) return rc;
    const long long blocks = (n + 255) / 256, cap = (long long)num_sms() * 8;
    k_cfl_maxima<<<(int)(blocks < cap ? blocks : cap), 256, 0, s>>>(n, rho, rhou, rhov, rhow, rhoY, gamm,
                                                                   1.0 / sqrt(Msq), d);
    if ((rc = cuda_check(cudaGetLastError(), "bella_cfl_maxima: launch")) != BELLA_OK) return rc;
    unsigned long long h[6];
    if ((rc = cuda_check(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "bella_cfl_maxima: copy")) !=
        BELLA_OK)
        return rc;
    if ((rc = cuda_check(cudaStreamSynchronize(s), "bella_cfl_maxima: synchronize")) != BELLA_OK) return rc;
    for (int k = 0; k < 6; ++k) {
        double v;
        memcpy(&v, &h[k], sizeof(v));
        out[k] = v;
    }
    return BELLA_OK;
}
