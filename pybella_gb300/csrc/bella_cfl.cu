// bella_cfl.cu -- the maxima of the reference's CFL time step (cfl.py:5-74) over
// the device state: |u|, |v|, |w| and |u|+c, |v|+c, |w|+c with the sound speed
// c = sqrt(gamma rhoY^gamma / rho) / sqrt(Msq), over every cell (ghosts included,
// as the reference takes .max() of the whole arrays).  One thread per cell, a
// block maximum, then an atomic maximum on the bit patterns (non-negative doubles
// order as their bit patterns do).  The time step itself is host arithmetic.
#include <cstring>

#include "bella_internal.cuh"

namespace bella {

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
        for (int k = 0; k < 6; ++k) m[k] = fmax(m[k], q[k]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 6; ++k) {
        double v = m[k];
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, red[threadIdx.x][w]);
        atomicMax(&out[threadIdx.x], (unsigned long long)__double_as_longlong(v));
    }
}

}  // namespace bella

using namespace bella;

extern "C" int bella_cfl_maxima(const double *rho, const double *rhou, const double *rhov, const double *rhow,
                                const double *rhoY, long long n, double gamm, double Msq, double *out, void *stream) {
    if (!rho || !rhou || !rhov || !rhow || !rhoY || !out || n <= 0 || Msq <= 0.0) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *d = nullptr;
    if (cudaMallocAsync(&d, 6 * sizeof(unsigned long long), s) != cudaSuccess) return BELLA_ECUDA;
    cudaMemsetAsync(d, 0, 6 * sizeof(unsigned long long), s);
    const long long blocks = (n + 255) / 256;
    k_cfl_maxima<<<(int)(blocks < NSM * 8 ? blocks : NSM * 8), 256, 0, s>>>(n, rho, rhou, rhov, rhow, rhoY, gamm,
                                                                         1.0 / sqrt(Msq), d);
    unsigned long long h[6];
    cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return BELLA_ECUDA;
    for (int k = 0; k < 6; ++k) {
        double v;
        memcpy(&v, &h[k], sizeof(v));
        out[k] = v;
    }
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}
