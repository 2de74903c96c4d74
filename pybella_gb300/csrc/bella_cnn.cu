// bella_cnn.cu -- the learned preconditioner's CNN on the tensor cores.
//
// Six 3x3x3 convolutions with zero padding, 1 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1
// channels, ReLU after the first five; BF16 weights and activations, FP32
// accumulation.  Every layer is an implicit GEMM
//   out[v, co] = sum_{tap, ci} in[v + off(tap), ci] * W[tap, ci, co]
// (M = voxels, N = output channels, K = 27 taps x input channels) run with
// mma.sync m16n8k16 BF16 tensor-core instructions.  A persistent CTA keeps the
// layer's weights in shared memory ([tap][co][ci], swizzled for ldmatrix) and
// loops over 4x4x16-voxel tiles: it stages the tile plus a one-voxel halo of
// the channels-last input (swizzled 16-byte chunks), each warp owns two 16-voxel
// rows along z and accumulates 16 x COUT in registers, then adds the bias,
// applies ReLU and stores BF16 (or FP32 for the last layer).  The input layer
// pads 1 channel to 16 and the output layer 1 channel to 8 (tensor-core shapes).
// Gradients for training: input gradients reuse the forward kernel with the
// taps mirrored and (ci, co) swapped; weight gradients are FP32 reductions on
// the CUDA cores.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "bella_internal.cuh"

namespace bella {

constexpr int CT_X = 4, CT_Y = 4, CT_Z = 16;                // output tile (voxels)
constexpr int CH_X = CT_X + 2, CH_Y = CT_Y + 2, CH_Z = CT_Z + 2;
constexpr int CH_VOX = CH_X * CH_Y * CH_Z;                    // 648 halo voxels
constexpr int CNN_THREADS = 256;                              // 8 warps x 2 m-tiles = 16 rows of 16 voxels

__device__ __forceinline__ int tap_of(int dx, int dy, int dz) { return (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1); }

// byte offset of (row, 16-byte chunk) in a swizzled [rows][CIN] bf16 array
template <int CIN>
__device__ __forceinline__ uint32_t swz(int row, int chunk) {
    constexpr int NCH = CIN / 8;             // 16-byte chunks per row (2 or 4)
    const int p = (NCH == 4) ? (chunk ^ ((row >> 1) & 3)) : (chunk ^ ((row >> 2) & 1));
    return (uint32_t)(row * (CIN * 2) + p * 16);
}

__device__ __forceinline__ void ldmatrix_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}

__device__ __forceinline__ void ldmatrix_x2(uint32_t addr, uint32_t &r0, uint32_t &r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                 "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Implicit-GEMM 3x3x3 convolution.  in: [nvox][CIN] bf16 (channels-last),
// W: [27][COUT][CIN] bf16, bias: [COUT] f32.  out: [nvox][COUT] bf16, or
// [nvox][COUT] f32 scaled by out_scale when OUTF32.
// FLIP mirrors the taps (input-gradient pass).  mask (optional, [nvox][COUT]
// bf16): the output is multiplied by (mask > 0) -- the ReLU derivative.
template <int CIN, int COUT, bool RELU, bool OUTF32, bool FLIP>
__global__ void __launch_bounds__(CNN_THREADS)
k_conv3d(int nx, int ny, int nz, int xseg, const __nv_bfloat16 *__restrict__ in, const __nv_bfloat16 *__restrict__ W,
         const float *__restrict__ bias, void *out, float out_scale, const __nv_bfloat16 *__restrict__ mask) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *sW = smem;                                   // 27 * COUT * CIN * 2 bytes
    unsigned char *sIn = smem + 27 * COUT * CIN * 2;            // CH_VOX * CIN * 2 bytes
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // weights -> shared memory (swizzled rows = (tap, co))
    for (int e = tid; e < 27 * COUT * (CIN / 8); e += CNN_THREADS) {
        const int row = e / (CIN / 8), ch = e - row * (CIN / 8);
        const uint4 v = *reinterpret_cast<const uint4 *>(W + (size_t)row * CIN + ch * 8);
        *reinterpret_cast<uint4 *>(sW + swz<CIN>(row, ch)) = v;
    }
    const int tx = (nx + CT_X - 1) / CT_X, ty = (ny + CT_Y - 1) / CT_Y, tz = (nz + CT_Z - 1) / CT_Z;
    const long long ntiles = (long long)tx * ty * tz;
    const uint32_t sW_base = (uint32_t)__cvta_generic_to_shared(sW);
    const uint32_t sIn_base = (uint32_t)__cvta_generic_to_shared(sIn);
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tzi = (int)(tile % tz);
        const long long rest = tile / tz;
        const int tyi = (int)(rest % ty), txi = (int)(rest / ty);
        const int i0 = txi * CT_X, j0 = tyi * CT_Y, k0 = tzi * CT_Z;
        __syncthreads();   // previous tile's reads of sIn are done (and sW is written)
        // halo tile of the input (zero outside the domain)
        for (int e = tid; e < CH_VOX * (CIN / 8); e += CNN_THREADS) {
            const int vox = e / (CIN / 8), ch = e - vox * (CIN / 8);
            const int la = vox / (CH_Y * CH_Z), rem = vox - la * (CH_Y * CH_Z), lb = rem / CH_Z, lc = rem - lb * CH_Z;
            const int gi = i0 - 1 + la, gj = j0 - 1 + lb, gk = k0 - 1 + lc;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            // a batch of crops lies along x in segments of xseg voxels (multiple of the tile
            // width): the halo never reaches into a neighbouring crop
            const bool same_seg = gi >= 0 && (gi / xseg) == (i0 / xseg);
            if (same_seg && gi < nx && gj >= 0 && gj < ny && gk >= 0 && gk < nz) {
                const size_t g = ((size_t)gi * ny + gj) * nz + gk;
                v = *reinterpret_cast<const uint4 *>(in + g * CIN + ch * 8);
            }
            *reinterpret_cast<uint4 *>(sIn + swz<CIN>(vox, ch)) = v;
        }
        __syncthreads();
        // warp -> two m-tiles (16 z-voxels each) of the 4x4 (x, y) rows
        float acc[2][COUT / 8][4];
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int n = 0; n < COUT / 8; ++n)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.f;
        const int rowA = (lane & 7) + ((lane >> 3) & 1) * 8;   // ldmatrix row supplied by this lane
        const int chA = lane >> 4;                              // k half supplied by this lane
#pragma unroll 1
        for (int tap = 0; tap < 27; ++tap) {
            const int dx = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dz = tap % 3 - 1;
            const int wtap = FLIP ? tap_of(-dx, -dy, -dz) : tap;
#pragma unroll
            for (int ks = 0; ks < CIN / 16; ++ks) {
                // B fragments for all n-tiles of this (tap, k-step)
                uint32_t b[COUT / 8][2];
                if (COUT >= 16) {
#pragma unroll
                    for (int np = 0; np < COUT / 16; ++np) {
                        const int brow = wtap * COUT + np * 16 + (lane & 7) + ((lane >> 4) & 1) * 8;
                        const int bch = ks * 2 + ((lane >> 3) & 1);
                        ldmatrix_x4(sW_base + swz<CIN>(brow, bch), b[2 * np][0], b[2 * np][1], b[2 * np + 1][0],
                                    b[2 * np + 1][1]);
                    }
                } else {
                    const int brow = wtap * COUT + (lane & 7);
                    const int bch = ks * 2 + ((lane >> 3) & 1);
                    ldmatrix_x2(sW_base + swz<CIN>(brow, bch), b[0][0], b[0][1]);
                }
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    const int mt = warp * 2 + m;                  // 0..15 -> (x, y) row of the tile
                    const int la = mt / CT_Y, lb = mt - la * CT_Y;
                    const int vox = ((la + 1 + dx) * CH_Y + (lb + 1 + dy)) * CH_Z + (1 + dz) + rowA;
                    uint32_t a0, a1, a2, a3;
                    ldmatrix_x4(sIn_base + swz<CIN>(vox, ks * 2 + chA), a0, a1, a2, a3);
#pragma unroll
                    for (int n = 0; n < COUT / 8; ++n) mma_bf16(acc[m][n], a0, a1, a2, a3, b[n][0], b[n][1]);
                }
            }
        }
        // epilogue: bias, ReLU (or ReLU-derivative mask), store
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int mt = warp * 2 + m;
            const int la = mt / CT_Y, lb = mt - la * CT_Y;
            const int gi = i0 + la, gj = j0 + lb;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                const int gk = k0 + (lane >> 2) + half * 8;
                if (gi >= nx || gj >= ny || gk >= nz) continue;
                const size_t g = ((size_t)gi * ny + gj) * nz + gk;
#pragma unroll
                for (int n = 0; n < COUT / 8; ++n) {
                    const int co = n * 8 + (lane & 3) * 2;
                    float v0 = acc[m][n][half * 2 + 0], v1 = acc[m][n][half * 2 + 1];
                    if (bias) { v0 += bias[co]; v1 += bias[co + 1]; }
                    if (RELU) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                    if (mask) {
                        const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(mask + g * COUT + co);
                        if (!(__bfloat162float(mk.x) > 0.f)) v0 = 0.f;
                        if (!(__bfloat162float(mk.y) > 0.f)) v1 = 0.f;
                    }
                    if (OUTF32) {
                        *reinterpret_cast<float2 *>(reinterpret_cast<float *>(out) + g * COUT + co) =
                            make_float2(v0 * out_scale, v1 * out_scale);
                    } else {
                        *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<__nv_bfloat16 *>(out) + g * COUT + co) =
                            __floats2bfloat162_rn(v0, v1);
                    }
                }
            }
        }
    }
}

template <int CIN, int COUT>
constexpr size_t conv_smem() { return (size_t)27 * COUT * CIN * 2 + (size_t)CH_VOX * CIN * 2; }

// ---------------------------------------------------------------------------
// The same convolution on the sm_100-family tensor-core path: tcgen05.mma with
// FP32 accumulators in tensor memory.  Rows of the GEMM are 128 consecutive
// positions of the zero-padded (y, z) plane of one x-plane, f = (y+1)*PZ + (z+1)
// with PZ = nz + 2: for tap (dx, dy, dz) the A operand is the same row set of
// input plane x+dx shifted by dy*PZ + dz rows, so every tap reads a canonical
// K-major operand straight from the staged planes (no im2col copy).  Staged
// layout per input plane: [16-byte channel chunk][row][8 channels]; the
// descriptor's LBO steps between the two chunks of a K=16 step, its SBO between
// groups of 8 rows.  Rows on the padding ring are computed and discarded.
// Work: the (block of TC_ROWS padded rows, x-plane) items are shared evenly among
// the CTAs (one per SM); a CTA's share is one or two runs of consecutive x-planes
// of one block (TC_MB accumulators of 128 rows); input plane p feeds output
// planes p+1, p, p-1 (taps dx = -1, 0, 1), so consecutive planes share inputs.
//
// The CTA is warp-specialised and its roles meet only on mbarriers, so the
// tensor cores never wait for a block-wide barrier:
//   * producer warps stage input planes into a ring of TC_SLOTS shared-memory
//     slots with 16-byte asynchronous copies (source size 0 fills the padding),
//     each waiting for its slot to be released by the MMAs that read it last;
//     the copies' own completion arrives on the slot's mbarrier (the producers
//     never wait for their data);
//   * one thread of the MMA warp issues each input plane's MMAs once the plane
//     has landed and the accumulators it starts are free, then commits them once,
//     to the input plane's entry of a ring of TC_DRING completion barriers, which
//     both frees the plane's slot and marks the output plane it completes;
//   * epilogue warps (one per 32 tensor-memory lanes of each row block) take each
//     completed output plane out of tensor memory, zero its columns, write it,
//     and release the accumulators to the MMA thread.
// Every wait is bounded (TC_SPIN_LIMIT polls): on time-out the CTA records an
// error, every role leaves its loop, the MMA thread waits (bounded) for its
// issued MMAs, and tensor memory is freed.
constexpr int TC_MB = 2;                    // 128-row accumulators per output plane
constexpr int TC_ROWS = 128 * TC_MB;
constexpr int TC_SLOTS = 5;                 // ring of staged input planes
constexpr int TC_DRING = 32;                // completion barriers of input planes: longer than any
                                            // waiter lags (input slots 5, 6 outputs in flight of up
                                            // to 3 inputs each), so no phase parity aliases
constexpr long long TC_SPIN_LIMIT = 1LL << 24;
constexpr size_t TC_SMEM_MAX = 225 * 1024;   // dynamic part; the kernel's static shared variables come on top
constexpr int TC_EPI_WARPS = 4 * TC_MB;      // warps 0 .. 7: epilogue, row block w / 4, lanes 32 * (w % 4)
constexpr int TC_PROD_WARPS = 3;             // warps 8 .. 10: producers
constexpr int TC_MMA_WARP = TC_EPI_WARPS + TC_PROD_WARPS;   // warp 11: tensor memory and the MMAs
constexpr int TC_THREADS = 32 * (TC_MMA_WARP + 1);

__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;                 // sm_100-family descriptor version; no swizzle
    return d;
}

template <int N>
__device__ __forceinline__ uint32_t tc_idesc() {   // kind::f16: BF16 x BF16 -> FP32, K-major A and B, M = 128
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ uint32_t tc_idesc_n(int n) {   // as tc_idesc<N> with N at run time
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

template <int CIN, int COUT>
__host__ __device__ constexpr size_t tc_smem_bytes(int pz) {
    return (size_t)9 * (CIN / 8) * 3 * COUT * 16 + (size_t)TC_SLOTS * (CIN / 8) * (TC_ROWS + 2 * pz + 2) * 16;
}

// bounded wait for the completion of the mbarrier phase of the given parity;
// gives up early when another role has set *abort
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, volatile int *abort) {
    for (long long it = 0; it < TC_SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.b32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(mbar), "r"(parity));
        if (done) return true;
        if ((it & 255) == 255 && *abort) return false;
    }
    return false;
}

// the same wait for a whole warp: lane 0 polls, every lane gets the result
__device__ __forceinline__ bool tc_wait_warp(uint32_t mbar, uint32_t parity, volatile int *abort) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = tc_wait(mbar, parity, abort) ? 1 : 0;
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void tc_arrive(uint32_t mbar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

// The work decomposition shared by all roles: the (row block, x-plane) items
// fb * nx + x, nblk * nx of them, are cut into one contiguous share of `work`
// items per CTA; a share is one or more runs, each covering row block fb and
// output x-planes [ia, ib) and reading input planes ia-1 .. ib.
struct TcRun {
    int fb, ia, ib;
};
__device__ __forceinline__ bool tc_next(long long &idx, long long hi, int nx, TcRun &r) {
    if (idx >= hi) return false;
    r.fb = (int)(idx / nx);
    r.ia = (int)(idx - (long long)r.fb * nx);
    r.ib = (int)min((long long)nx, (long long)r.ia + (hi - idx));
    idx += r.ib - r.ia;
    return true;
}

// Input plane p feeds output planes p+1, p, p-1 through the weights of taps dx = 0, 1, 2:
// with the three taps side by side in B (N = 96) one MMA per (dy, dz, K-step) serves
// all three output planes.  Output planes are numbered o = 0, 1, ... in the order the
// CTA produces them; a row block's accumulators are TC_RING blocks of COUT
// tensor-memory columns, and at most TC_LIVE output planes hold accumulators at a
// time.  The MMAs of the input plane whose output window is w, w-1, w-2 (w the index
// of plane p+1) write blocks b, b+1, b+2 with b = tc_win(w) = (1 - w) mod TC_LIVE, so a
// window never wraps (b + 2 <= 7) and every input plane is one MMA per (tap, K-step).
// Output o, a = -o mod TC_LIVE, then collects its contributions in block a+1, except
// for a = 0 (block 1 from planes o-1 and o, block 7 from o+1) and a = TC_LIVE-1 (block 0
// from o-1, block 6 from o and o+1): the epilogue adds the two blocks (tc_blocks).
// Only outputs o +- k*TC_LIVE share blocks, so output o may start once the epilogue has
// released output o - TC_LIVE.  Every block is zeroed by its epilogue and every MMA
// accumulates.  Output planes outside the run or in another sample's x-segment are
// left out of an MMA's column range (a sub-range of the window).
constexpr int TC_RING = 8;                   // accumulator blocks per row block
constexpr int TC_LIVE = 6;                   // output planes holding accumulators at a time

__host__ __device__ __forceinline__ int tc_win(long long w) {
    return (int)(((1 - w) % TC_LIVE + TC_LIVE) % TC_LIVE);
}
// the accumulator blocks of output o: primary, and the second one or -1
__host__ __device__ __forceinline__ void tc_blocks(long long o, int &pb, int &sb) {
    const int a = (int)(((-o) % TC_LIVE + TC_LIVE) % TC_LIVE);
    pb = a == TC_LIVE - 1 ? TC_LIVE : a + 1;
    sb = a == 0 ? TC_LIVE + 1 : (a == TC_LIVE - 1 ? 0 : -1);
}

// COUT = 32: hidden layers, BF16 output with bias and optional ReLU.  COUT = 16 with
// OUTF32: the output layer (8 channels padded to 16), FP32 output (acc + bias) *
// out_scale of its first 8 channels.
template <int CIN, int COUT, bool RELU, bool OUTF32>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_conv3d_tc(int nx, int ny, int nz, int xseg, long long work, const __nv_bfloat16 *__restrict__ in,
            const __nv_bfloat16 *__restrict__ Wtc, const float *__restrict__ bias, void *out, float out_scale,
            int *err, const __nv_bfloat16 *__restrict__ mask) {
    static_assert(COUT == 32 || (COUT == 16 && OUTF32), "hidden layers: 32 channels; output layer: 16 (8 used)");
    // the next layer, launched as a programmatic dependent, may start its prologue
    // on the SMs this grid leaves (it waits for this grid before it touches activations)
    asm volatile("griddepcontrol.launch_dependents;");
    constexpr int TMEM_COLS = TC_MB * TC_RING * COUT;     // 512 or 256: a power of two
    constexpr int NCH = CIN / 8;
    constexpr int NB = 3 * COUT;                          // B rows: the three dx taps
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar_full[TC_SLOTS], bar_mma[TC_DRING], bar_free[TC_LIVE];
    __shared__ __align__(8) uint64_t bar_done;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    volatile int *abort = &abort_flag;
    const int PZ = nz + 2, PY = ny + 2;
    const int L = TC_ROWS + 2 * PZ + 2;                   // staged rows per plane and chunk
    unsigned char *sW = smem;                             // [9][NCH][3*COUT][16 B]
    unsigned char *sA = smem + (size_t)9 * NCH * NB * 16; // [TC_SLOTS][NCH][L][16 B]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    auto sa = [](const void *p) { return (uint32_t)__cvta_generic_to_shared(p); };
    for (int e = tid; e < 9 * NCH * NB; e += TC_THREADS)      // the weights, all copies in flight at once
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa(sW) + 16u * e),
                     "l"(reinterpret_cast<const uint4 *>(Wtc) + e));
    asm volatile("cp.async.commit_group;");
    asm volatile("cp.async.wait_group 0;");
    asm volatile("fence.proxy.async.shared::cta;");     // the weights are read by the tensor cores
    if (tid == 0) {
        for (int k = 0; k < TC_SLOTS; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(&bar_full[k])), "r"(32 * TC_PROD_WARPS));
        for (int k = 0; k < TC_DRING; ++k) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(&bar_mma[k])));
        for (int k = 0; k < TC_LIVE; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(&bar_free[k])), "r"(TC_EPI_WARPS));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(&bar_done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        abort_flag = 0;
    }
    if (warp == TC_MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sa(&tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    auto zero_cols = [&](uint32_t taddr) {
        const uint32_t z = 0u;
        if (COUT == 32)
            asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
                         "{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,"
                         "%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(z));
        else
            asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
                         "{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(z));
    };
    // epilogue warp w owns lanes 32*(w%4) of row block w/4: zero its accumulator ring
    const uint32_t tlane = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((warp >> 2) * TC_RING * COUT);
    if (warp < TC_EPI_WARPS) {
        for (int q = 0; q < TC_RING; ++q) zero_cols(tlane + (uint32_t)(q * COUT));
        asm volatile("tcgen05.wait::st.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // the prologue above touches only this layer's weights and on-chip state; the
    // input activations are the previous grid's output: wait for it to complete
    // (a no-op when this grid was not launched as a programmatic dependent)
    asm volatile("griddepcontrol.wait;" ::: "memory");

    const int plane = PY * PZ;
    const int nblk = (plane + TC_ROWS - 1) / TC_ROWS;
    const long long share_lo = (long long)blockIdx.x * work;
    const long long share_hi = min(share_lo + work, (long long)nblk * nx);
    const uint32_t sW_a = sa(sW), sA_a = sa(sA);

    if (warp >= TC_EPI_WARPS && warp < TC_MMA_WARP) {
        // ---------------- producers: input planes into the slot ring ----------------
        const int ptid = tid - 32 * TC_EPI_WARPS;
        const float inv_pz = 1.0f / (float)PZ;
        long long i = 0;                                  // input planes staged so far (this CTA)
        bool ok = true;
        long long idx = share_lo;
        TcRun R;
        while (ok && tc_next(idx, share_hi, nx, R)) {
            const int f0 = R.fb * TC_ROWS - (PZ + 1);     // padded row of staged row 0
            for (int p = R.ia - 1; p <= R.ib && ok; ++p, ++i) {
                const int slot = (int)(i % TC_SLOTS);
                const long long prev = i - TC_SLOTS;      // the slot's previous plane: its MMAs done?
                if (prev >= 0 &&
                    !tc_wait_warp(sa(&bar_mma[prev % TC_DRING]), (uint32_t)((prev / TC_DRING) & 1), abort)) {
                    ok = false;
                    break;
                }
                if (p >= 0 && p < nx) {
                    const uint32_t base = sA_a + (uint32_t)((size_t)slot * NCH * L * 16);
                    for (int rb = ptid; rb < L; rb += 32 * TC_PROD_WARPS) {
                        const int f = f0 + rb;
                        const __nv_bfloat16 *src = in;
                        uint32_t bytes = 0;
                        if (f >= 0 && f < plane) {
                            int yq = __float2int_rz((float)f * inv_pz);   // f / PZ to within one (f < 2^24)
                            int zr = f - yq * PZ;
                            if (zr < 0) { --yq; zr += PZ; } else if (zr >= PZ) { ++yq; zr -= PZ; }
                            const int y = yq - 1, z = zr - 1;
                            if (y >= 0 && y < ny && z >= 0 && z < nz) {
                                src = in + (((size_t)p * ny + y) * nz + z) * CIN;
                                bytes = 16;
                            }
                        }
#pragma unroll
                        for (int ch = 0; ch < NCH; ++ch)
                            asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                                         ::"r"(base + (uint32_t)((ch * L + rb) * 16)), "l"(src + (bytes ? ch * 8 : 0)),
                                           "r"(bytes));
                    }
                }
                // arrives on the slot's barrier once this thread's copies so far have landed
                asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(sa(&bar_full[slot])));
            }
        }
        asm volatile("cp.async.wait_all;");
        if (!ok && ptid == 0) {
            atomicExch(err, 1);
            *abort = 1;
        }
    } else if (warp == TC_MMA_WARP) {
        // ---------------- one thread issues the MMAs ----------------
        if (lane == 0) {
            const uint64_t a0 = tc_sdesc(sA_a, (uint32_t)L * 16, 128), b0 = tc_sdesc(sW_a, NB * 16, 128);
            long long i = 0, obase = 0, acq = 0;
            bool ok = true;
            // the MMAs of input plane p (ring slot `slot`) into n output planes from ohi
            // down, at accumulator blocks blk, blk+1, ...; plane ohi uses the dx tap d0
            auto mma_range = [&](int slot, int blk, int n, int d0) {
                const uint32_t col = (uint32_t)(COUT * blk);
                const uint32_t idesc = tc_idesc_n(n * COUT);
                const uint64_t abase = a0 + (uint64_t)(slot * NCH * L + PZ + 1);
#pragma unroll
                for (int mb = 0; mb < TC_MB; ++mb) {
                    const uint32_t dtm = tmem + (uint32_t)(mb * TC_RING * COUT) + col;
#pragma unroll
                    for (int dyi = 0; dyi < 3; ++dyi) {
#pragma unroll
                        for (int dzi = 0; dzi < 3; ++dzi) {
                            const int t9 = dyi * 3 + dzi;
#pragma unroll
                            for (int ks = 0; ks < CIN / 16; ++ks) {
                                const uint64_t ad =
                                    abase + (uint64_t)(mb * 128 + 2 * ks * L + (dyi - 1) * PZ + (dzi - 1));
                                const uint64_t bd = b0 + (uint64_t)((t9 * NCH + 2 * ks) * NB + COUT * d0);
                                asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                                             ::"r"(dtm), "l"(ad), "l"(bd), "r"(idesc), "r"(1));
                            }
                        }
                    }
                }
            };
            long long idx = share_lo;
            TcRun R;
            while (ok && tc_next(idx, share_hi, nx, R)) {
                for (int p = R.ia - 1; p <= R.ib; ++p, ++i) {
                    const int slot = (int)(i % TC_SLOTS);
                    if (!tc_wait(sa(&bar_full[slot]), (uint32_t)((i / TC_SLOTS) & 1), abort)) {
                        ok = false;
                        break;
                    }
                    asm volatile("fence.proxy.async.shared::cta;");
                    if (p >= 0 && p < nx) {
                        const int s0 = (p / xseg) * xseg;     // this sample's x-segment
                        const int qlo = max(max(p - 1, R.ia), s0), qhi = min(min(p + 1, R.ib - 1), s0 + xseg - 1);
                        if (qlo <= qhi) {
                            const long long olo = obase + (qlo - R.ia), ohi = obase + (qhi - R.ia);
                            for (; acq <= ohi && ok; ++acq)   // output acq - TC_LIVE released its blocks?
                                if (acq >= TC_LIVE &&
                                    !tc_wait(sa(&bar_free[acq % TC_LIVE]), (uint32_t)((acq / TC_LIVE - 1) & 1), abort))
                                    ok = false;
                            if (!ok) break;
                            asm volatile("tcgen05.fence::after_thread_sync;");
                            const int d0 = p + 1 - qhi;           // dx tap of plane qhi
                            const long long w = obase + (p + 1 - R.ia);   // the window's first output
                            mma_range(slot, tc_win(w) + (int)(w - ohi), (int)(ohi - olo + 1), d0);
                        }
                    }
                    // one commit: the slot is free and output plane p-1 complete once these MMAs are done
                    tc_commit(sa(&bar_mma[i % TC_DRING]));
                }
                obase += R.ib - R.ia;
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort = 1;
            }
            tc_commit(sa(&bar_done));                         // every MMA issued above has completed
            int never = 0;                                    // (this wait does not give up on an abort)
            if (!tc_wait(sa(&bar_done), 0u, &never)) atomicExch(err, 1);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue warps ----------------
        const int mb = warp >> 2;
        long long o = 0, ibase = 0;                       // output planes done; input index of the run's first
        bool ok = true;
        long long idx = share_lo;
        TcRun R;
        while (ok && tc_next(idx, share_hi, nx, R)) {
            for (int q = R.ia; q < R.ib; ++q, ++o) {
                const long long j = ibase + (q - R.ia + 2);  // input plane q+1 completes output plane q
                if (!tc_wait_warp(sa(&bar_mma[j % TC_DRING]), (uint32_t)((j / TC_DRING) & 1), abort)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                int pb, sb;
                tc_blocks(o, pb, sb);
                const uint32_t taddr = tlane + (uint32_t)(COUT * pb);
                uint32_t r[32];
                if (COUT == 32)
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
                                   "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
                                   "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
                                   "=r"(r[31])
                                 : "r"(taddr));
                else
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                                 : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                zero_cols(taddr);                           // the block's next plane accumulates from zero
                if (sb >= 0) {                              // the contributions in the second block
                    const uint32_t saddr = tlane + (uint32_t)(COUT * sb);
#pragma unroll
                    for (int h = 0; h < COUT; h += 16) {
                        uint32_t t[16];
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                                     "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                                     : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]),
                                       "=r"(t[6]), "=r"(t[7]), "=r"(t[8]), "=r"(t[9]), "=r"(t[10]), "=r"(t[11]),
                                       "=r"(t[12]), "=r"(t[13]), "=r"(t[14]), "=r"(t[15])
                                     : "r"(saddr + (uint32_t)h));
                        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                        for (int c = 0; c < 16; ++c)
                            r[h + c] = __float_as_uint(__uint_as_float(r[h + c]) + __uint_as_float(t[c]));
                    }
                    zero_cols(saddr);
                }
                const int f = R.fb * TC_ROWS + mb * 128 + (warp & 3) * 32 + lane;
                if (f < plane) {
                    const int yq = f / PZ;
                    const int y = yq - 1, z = f - yq * PZ - 1;
                    if (y >= 0 && y < ny && z >= 0 && z < nz) {
                        const size_t g = ((size_t)q * ny + y) * nz + z;
                        if (OUTF32) {                        // the output layer's 8 real channels
                            float v[8];
#pragma unroll
                            for (int c = 0; c < 8; ++c)
                                v[c] = (__uint_as_float(r[c]) + (bias ? bias[c] : 0.f)) * out_scale;
                            float4 *ov = reinterpret_cast<float4 *>(reinterpret_cast<float *>(out) + g * 8);
                            ov[0] = make_float4(v[0], v[1], v[2], v[3]);
                            ov[1] = make_float4(v[4], v[5], v[6], v[7]);
                        } else {
                            uint32_t w[16], mk[16];
                            if (mask) {                  // ReLU derivative of the input-gradient pass
                                const uint4 *mv = reinterpret_cast<const uint4 *>(mask + g * COUT);
#pragma unroll
                                for (int c4 = 0; c4 < 4; ++c4) {
                                    const uint4 t = mv[c4];
                                    mk[4 * c4] = t.x; mk[4 * c4 + 1] = t.y; mk[4 * c4 + 2] = t.z; mk[4 * c4 + 3] = t.w;
                                }
                            }
#pragma unroll
                            for (int c = 0; c < 16; ++c) {
                                float v0 = __uint_as_float(r[2 * c]), v1 = __uint_as_float(r[2 * c + 1]);
                                if (bias) { v0 += bias[2 * c]; v1 += bias[2 * c + 1]; }
                                if (RELU) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                                if (mask) {
                                    const __nv_bfloat162 m2 = *reinterpret_cast<const __nv_bfloat162 *>(&mk[c]);
                                    if (!(__bfloat162float(m2.x) > 0.f)) v0 = 0.f;
                                    if (!(__bfloat162float(m2.y) > 0.f)) v1 = 0.f;
                                }
                                const __nv_bfloat162 h2 = __floats2bfloat162_rn(v0, v1);
                                w[c] = *reinterpret_cast<const uint32_t *>(&h2);
                            }
                            uint4 *ov = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(out) + g * COUT);
                            ov[0] = make_uint4(w[0], w[1], w[2], w[3]);
                            ov[1] = make_uint4(w[4], w[5], w[6], w[7]);
                            ov[2] = make_uint4(w[8], w[9], w[10], w[11]);
                            ov[3] = make_uint4(w[12], w[13], w[14], w[15]);
                        }
                    }
                }
                asm volatile("tcgen05.wait::st.sync.aligned;");
                asm volatile("tcgen05.fence::before_thread_sync;");
                __syncwarp();
                if (lane == 0) tc_arrive(sa(&bar_free[o % TC_LIVE]));
            }
            ibase += R.ib - R.ia + 2;                     // the run read input planes ia-1 .. ib
        }
        if (!ok && lane == 0) {
            atomicExch(err, 1);
            *abort = 1;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == TC_MMA_WARP)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// kernel weights [27][COUTP][CINP] (tap = (dx+1)*9 + (dy+1)*3 + (dz+1)) -> tensor-core
// operand order [dy,dz][CINP/8][dx][COUTD][8] (COUTD >= COUTP; rows past COUTP are
// zero): for each (dy, dz) and 8-channel chunk, the three dx taps' output channels
// are 3*COUTD consecutive B rows
// flip: read the mirrored tap (-dx, -dy, -dz), i.e. 26 - tap (the input-gradient pass)
__global__ void k_wk_to_tc(const __nv_bfloat16 *wk, int cinp, int coutp, int coutd, __nv_bfloat16 *wtc, int flip) {
    const int total = 27 * cinp * coutd;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int tap = e / (cinp * coutd), r = e - tap * cinp * coutd, co = r / cinp, ci = r - co * cinp;
        const int dx = tap / 9, t9 = tap - dx * 9;
        const int src = flip ? 26 - tap : tap;
        const __nv_bfloat16 v = co < coutp ? wk[((size_t)src * coutp + co) * cinp + ci] : __float2bfloat16(0.f);
        wtc[((((size_t)t9 * (cinp / 8) + ci / 8) * 3 + dx) * coutd + co) * 8 + (ci % 8)] = v;
    }
}

// Node grid <-> net grid.  Samples are stacked along x: node (s, i, j, k) of a
// [B][nx][ny][nz] array maps to net voxel ((s*cx + i/b)*cy + j/b)*cz + k/b and
// sub-node channel ((i%b)*b + j%b)*b + k%b, with cx = ceil(nx/b) etc.
struct BlockMap {
    int B, nx, ny, nz, b, cx, cy, cz;
    __host__ __device__ long long nvox() const { return (long long)B * cx * cy * cz; }
};

static BlockMap make_map(int B, int nx, int ny, int nz, int b) {
    return BlockMap{B, nx, ny, nz, b, (nx + b - 1) / b, (ny + b - 1) / b, (nz + b - 1) / b};
}

// scale of a unit-RMS normalisation from a device sum of squares of nn values
__device__ __forceinline__ float rms_scale(const double *sumsq, long long nn) {
    const double q = *sumsq;
    return (q > 0.0 && isfinite(q)) ? (float)(1.0 / sqrt(q / (double)nn)) : 1.f;
}

// voxel v of the net grid -> (sample, ci, cj, ck); 32-bit (node and voxel counts
// stay below 2^31: bella_cnn_create bounds the capacity)
struct VoxIdx {
    int s, ci, cj, ck;
};
__device__ __forceinline__ VoxIdx vox_index(const BlockMap &m, int v) {
    VoxIdx r;
    r.ck = v % m.cz;
    const int t = v / m.cz;
    r.cj = t % m.cy;
    const int sx = t / m.cy;
    r.s = sx / m.cx;
    r.ci = sx - r.s * m.cx;
    return r;
}

// node values (f32, times scale -- or 1/RMS from sumsq when given) -> channels-last
// bf16 with 16 channels; one thread per voxel, BB = m.b (1 or 2) at compile time
template <int BB>
__global__ void k_pack_in(BlockMap m, const float *in, float scale, __nv_bfloat16 *out, const double *sumsq) {
    const int n = (int)m.nvox();
    if (sumsq) scale = rms_scale(sumsq, (long long)m.B * m.nx * m.ny * m.nz);
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const VoxIdx x = vox_index(m, v);
        float c[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) c[q] = 0.f;
#pragma unroll
        for (int q = 0; q < BB * BB * BB; ++q) {
            const int a = q / (BB * BB), bb = (q / BB) % BB, d = q % BB;
            const int i = x.ci * BB + a, j = x.cj * BB + bb, k = x.ck * BB + d;
            if (i < m.nx && j < m.ny && k < m.nz)
                c[q] = in[((x.s * m.nx + i) * m.ny + j) * m.nz + k] * scale;
        }
        uint32_t w[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(c[2 * q], c[2 * q + 1]);
            w[q] = *reinterpret_cast<const uint32_t *>(&h);
        }
        uint4 *o = reinterpret_cast<uint4 *>(out + (long long)v * 16);
        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// node values (f32) -> net-grid f32 with 8 channels (training targets, output gradients)
__global__ void k_pack_f32(BlockMap m, const float *in, float scale, float *out) {
    const long long n = m.nvox();
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int ck = (int)(v % m.cz);
        const long long t = v / m.cz;
        const int cj = (int)(t % m.cy);
        const long long sx = t / m.cy;
        const int s = (int)(sx / m.cx), ci = (int)(sx % m.cx);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            float c = 0.f;
            if (q < m.b * m.b * m.b) {
                const int a = q / (m.b * m.b), bb = (q / m.b) % m.b, d = q % m.b;
                const int i = ci * m.b + a, j = cj * m.b + bb, k = ck * m.b + d;
                if (i < m.nx && j < m.ny && k < m.nz) c = in[(((long long)s * m.nx + i) * m.ny + j) * m.nz + k] * scale;
            }
            out[v * 8 + q] = c;
        }
    }
}

// net-grid f32 [nvox][8] -> node values (times RMS from sumsq when given), plus
// omega * skip (the identity path of the preconditioner) when skip is given
// seam: the network's reach in nodes; along an axis flagged in pmask (bit 0 x, 1 y,
// 2 z) the output is 0 within that distance of the duplicated periodic seam.
// One thread per voxel: its 8 channels in two 16-byte loads, its BB^3 nodes
// written as z pairs (coalesced across the warp); BB = m.b at compile time.
template <int BB>
__global__ void k_unpack(BlockMap m, const float *y8, float *out, const double *sumsq, const float *skip = nullptr,
                         float omega = 0.f, int pmask = 0, int seam = 0) {
    const int nv = (int)m.nvox();
    const float mul = sumsq ? 1.f / rms_scale(sumsq, (long long)m.B * m.nx * m.ny * m.nz) : 1.f;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const VoxIdx x = vox_index(m, v);
        const float4 lo = reinterpret_cast<const float4 *>(y8)[2 * (long long)v];
        const float4 hi = reinterpret_cast<const float4 *>(y8)[2 * (long long)v + 1];
        const float yv[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
        for (int q = 0; q < BB * BB * BB; ++q) {
            const int a = q / (BB * BB), bb = (q / BB) % BB, d = q % BB;
            const int i = x.ci * BB + a, j = x.cj * BB + bb, k = x.ck * BB + d;
            if (i >= m.nx || j >= m.ny || k >= m.nz) continue;
            const int e = ((x.s * m.nx + i) * m.ny + j) * m.nz + k;
            float o = yv[q] * mul;
            if (skip) o = fmaf(omega, skip[e], o);
            if (pmask) {
                const bool near = ((pmask & 1) && min(i, m.nx - 1 - i) < seam) ||
                                  ((pmask & 2) && min(j, m.ny - 1 - j) < seam) ||
                                  ((pmask & 4) && min(k, m.nz - 1 - k) < seam);
                if (near) o = 0.f;
            }
            out[e] = o;
        }
    }
}

// host launchers of the two, for the map's blocking factor (1 or 2)
static void pack_in(const BlockMap &m, const float *in, float scale, __nv_bfloat16 *out, const double *sumsq,
                    cudaStream_t s) {
    const int g = vec_grid(m.nvox());
    if (m.b == 2) k_pack_in<2><<<g, 256, 0, s>>>(m, in, scale, out, sumsq);
    else          k_pack_in<1><<<g, 256, 0, s>>>(m, in, scale, out, sumsq);
}
static void unpack(const BlockMap &m, const float *y8, float *out, const double *sumsq, const float *skip,
                   float omega, int pmask, int seam, cudaStream_t s) {
    const int g = vec_grid(m.nvox());
    if (m.b == 2) k_unpack<2><<<g, 256, 0, s>>>(m, y8, out, sumsq, skip, omega, pmask, seam);
    else          k_unpack<1><<<g, 256, 0, s>>>(m, y8, out, sumsq, skip, omega, pmask, seam);
}

// f32 [nvox][8] -> bf16 [nvox][16] (zero-padded), input of the last layer's gradient pass
__global__ void k_g8_to_bf16(long long n, const float *g8, __nv_bfloat16 *g16) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4 *>(g8)[2 * v], b = reinterpret_cast<const float4 *>(g8)[2 * v + 1];
        __nv_bfloat162 h[4] = {__floats2bfloat162_rn(a.x, a.y), __floats2bfloat162_rn(a.z, a.w),
                               __floats2bfloat162_rn(b.x, b.y), __floats2bfloat162_rn(b.z, b.w)};
        uint4 *o = reinterpret_cast<uint4 *>(g16 + v * 16);
        o[0] = *reinterpret_cast<uint4 *>(h);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// ---- training kernels (FP32 on the CUDA cores) ------------------------------------
// Weight gradients dW[tap][ci][co] = sum_v in[v + off(tap)][ci] * g[v][co] and bias
// gradients db[co] = sum_v g[v][co].  A persistent CTA stages a 4x4x16 tile of the
// gradient and the one-voxel halo of the input in shared memory (FP32) and keeps
// the 27 taps x (its ci, co pairs) in registers; partial sums are added to the
// global gradient once per CTA.
template <int CIN, int CINR, int COUT, int COUTR, typename GT>
__global__ void __launch_bounds__(256)
k_wgrad(int nx, int ny, int nz, int xseg, const __nv_bfloat16 *__restrict__ in, const GT *__restrict__ g,
        float *dW, float *db) {
    extern __shared__ __align__(16) float fsm[];
    float *sIn = fsm;                         // [CH_VOX][CINR]
    float *sG = fsm + CH_VOX * CINR;          // [256][COUTR]
    constexpr int NP = CINR * COUTR;          // (ci, co) pairs
    constexpr int PPT = (NP + 255) / 256;     // pairs per thread
    const int tid = threadIdx.x;
    float acc[PPT][27];
    float accb[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        accb[q] = 0.f;
#pragma unroll
        for (int t = 0; t < 27; ++t) acc[q][t] = 0.f;
    }
    const int tx = (nx + CT_X - 1) / CT_X, ty = (ny + CT_Y - 1) / CT_Y, tz = (nz + CT_Z - 1) / CT_Z;
    const long long ntiles = (long long)tx * ty * tz;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int tzi = (int)(tile % tz);
        const long long rest = tile / tz;
        const int tyi = (int)(rest % ty), txi = (int)(rest / ty);
        const int i0 = txi * CT_X, j0 = tyi * CT_Y, k0 = tzi * CT_Z;
        __syncthreads();
        for (int e = tid; e < CH_VOX * CINR; e += 256) {
            const int vox = e / CINR, ci = e - vox * CINR;
            const int la = vox / (CH_Y * CH_Z), rem = vox - la * (CH_Y * CH_Z), lb = rem / CH_Z, lc = rem - lb * CH_Z;
            const int gi = i0 - 1 + la, gj = j0 - 1 + lb, gk = k0 - 1 + lc;
            float v = 0.f;
            if (gi >= 0 && (gi / xseg) == (i0 / xseg) && gi < nx && gj >= 0 && gj < ny && gk >= 0 && gk < nz)
                v = __bfloat162float(in[(((size_t)gi * ny + gj) * nz + gk) * CIN + ci]);
            sIn[e] = v;
        }
        for (int e = tid; e < 256 * COUTR; e += 256) {
            const int vox = e / COUTR, co = e - vox * COUTR;
            const int la = vox / (CT_Y * CT_Z), rem = vox - la * (CT_Y * CT_Z), lb = rem / CT_Z, lc = rem - lb * CT_Z;
            const int gi = i0 + la, gj = j0 + lb, gk = k0 + lc;
            float v = 0.f;
            if (gi < nx && gj < ny && gk < nz) {
                const size_t gg = (((size_t)gi * ny + gj) * nz + gk) * COUT + co;
                if constexpr (sizeof(GT) == 2) v = __bfloat162float(g[gg]); else v = (float)g[gg];
            }
            sG[e] = v;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const int pr = tid + q * 256;
            if (pr >= NP) break;
            const int ci = pr / COUTR, co = pr - ci * COUTR;
            for (int vox = 0; vox < 256; ++vox) {
                const int la = vox / (CT_Y * CT_Z), rem = vox - la * (CT_Y * CT_Z), lb = rem / CT_Z, lc = rem - lb * CT_Z;
                const float gv = sG[vox * COUTR + co];
                accb[q] += gv;
                const int hb = ((la + 1) * CH_Y + (lb + 1)) * CH_Z + (lc + 1);
#pragma unroll
                for (int t = 0; t < 27; ++t) {
                    const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
                    acc[q][t] = fmaf(sIn[(hb + (dx * CH_Y + dy) * CH_Z + dz) * CINR + ci], gv, acc[q][t]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const int pr = tid + q * 256;
        if (pr >= NP) break;
        const int ci = pr / COUTR, co = pr - ci * COUTR;
#pragma unroll
        for (int t = 0; t < 27; ++t) atomicAdd(&dW[((size_t)t * CINR + ci) * COUTR + co], acc[q][t]);
        if (ci == 0 && db) atomicAdd(&db[co], accb[q]);
    }
}

template <int CINR, int COUTR>
constexpr size_t wgrad_smem() { return sizeof(float) * ((size_t)CH_VOX * CINR + 256 * COUTR); }

// ---- weight gradients on tcgen05 ---------------------------------------------------
// dW[t][ci][co] = sum_v in[v + off(t)][ci] g[v][co] as a GEMM whose K runs over voxels.
// Items are (x-plane q of the gradient, block of WG_ROWS padded (y, z) rows f0 ..);
// each CTA (one per SM) takes a contiguous share.  With w = f + dz the in-plane sum
// is sum_w in[w + dy*PZ][ci] g[w - dz][co], so per item a stage holds
//   * A: input planes q-1, q, q+1 in the forward kernel's layout ([16-byte channel
//     chunk][row][8 channels]), rows f0-8-PZ .. f0+WG_K-8+PZ-1 of the zero-padded
//     plane, zeros outside the plane and the sample's x-segment.  Read MN-major (a
//     chunk's 8 channels contiguous, rows 16 bytes apart), 16 consecutive chunks are
//     one operand of 128 rows (plane q-1+s, channel); rows past plane q+1 read other
//     data and are discarded.  For dy the operand starts dy*PZ rows later.
//   * B: three copies of the gradient rows of plane q, copy dz shifted by dz rows
//     (row w of copy dz is g[f0-8+w-dz], zero outside the item's rows): with the
//     copies' chunks in sequence, one MN-major operand of N = 3*COUT covers dz = -1..1.
// K = WG_K rows (WG_ROWS and 8 on either side), so three MMAs (dy) of N = 3*COUT per
// 16 rows; their accumulators (tap (dy, dz) at column ((dy+1)*3 + dz+1)*COUT) collect
// every item of the CTA and are added into dW once.  Three stages where they fit in
// shared memory (else two): the copies of the next items overlap the MMAs of this one.
constexpr int WG_THREADS = 256;
constexpr int WG_ROWS = 128;                // gradient rows per item
constexpr int WG_K = WG_ROWS + 16;          // K rows per item
constexpr int WG_CHUNKS = 16;               // 16-byte chunks of one A operand
constexpr int WG_MAX_STAGES = 3;

__host__ __device__ constexpr uint32_t wg_stage_bytes(int cin, int cout, int pz) {
    return (uint32_t)(((3 * (cin / 8) * (WG_K + 2 * pz) * 16 + 3 * (cout / 8) * WG_K * 16) >
                               WG_CHUNKS * (WG_K + 2 * pz) * 16
                           ? 3 * (cin / 8) * (WG_K + 2 * pz) * 16 + 3 * (cout / 8) * WG_K * 16
                           : WG_CHUNKS * (WG_K + 2 * pz) * 16) + 127) & ~127u;
}
// stages that fit the shared memory (at least two are needed)
__host__ __device__ constexpr int wg_stages(int cin, int cout, int pz) {
    return (size_t)WG_MAX_STAGES * wg_stage_bytes(cin, cout, pz) <= TC_SMEM_MAX ? WG_MAX_STAGES : 2;
}
__host__ __device__ constexpr size_t wg_smem_bytes(int cin, int cout, int pz) {
    return (size_t)wg_stages(cin, cout, pz) * wg_stage_bytes(cin, cout, pz);
}

template <int CIN, int COUT, int CINR, int COUTR>
__global__ void __launch_bounds__(WG_THREADS, 1)
k_wgrad_tc(int nx, int ny, int nz, int xseg, long long work, int nst, const __nv_bfloat16 *__restrict__ in,
           const __nv_bfloat16 *__restrict__ g, float *dW, int *err) {
    static_assert(CIN == 16 || CIN == 32, "input channels: 16 or 32");
    static_assert(COUT == 16 || COUT == 32, "gradient channels: 16 or 32");
    constexpr int NCH = CIN / 8, NCG = COUT / 8;
    constexpr int TMEM_COLS = 9 * COUT <= 256 ? 256 : 512;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar_mma[WG_MAX_STAGES];
    __shared__ __align__(8) uint64_t bar_done;
    __shared__ uint32_t tmem_slot;
    __shared__ int never;                                 // the waits here are not cut short by another role
    const int PZ = nz + 2, PY = ny + 2;
    const int L = WG_K + 2 * PZ;                          // staged input rows per chunk
    const uint32_t CS = (uint32_t)L * 16, CSB = (uint32_t)WG_K * 16;
    const uint32_t SS = wg_stage_bytes(CIN, COUT, PZ);
    const uint32_t BOFF = 3u * NCH * CS;                  // B after the three input planes
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    auto sa = [](const void *p) { return (uint32_t)__cvta_generic_to_shared(p); };
    const uint32_t s0 = sa(smem);
    if (tid == 0) {
        for (int k = 0; k < WG_MAX_STAGES; ++k)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(&bar_mma[k])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(&bar_done)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        never = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sa(&tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    const int plane = PY * PZ;
    const int nblk = (plane + WG_ROWS - 1) / WG_ROWS;
    const long long lo = (long long)blockIdx.x * work;
    const long long n_it = max(0LL, min(lo + work, (long long)nblk * nx) - lo);

    // row f of the padded plane -> (y, z) of the grid, false on the padding ring or outside
    const float inv_pz = 1.0f / (float)PZ;
    auto interior = [&](int f, int &y, int &z) {
        if (f < 0 || f >= plane) return false;
        int yq = __float2int_rz((float)f * inv_pz);       // exact to within one (f < 2^24)
        int r = f - yq * PZ;
        if (r < 0) { --yq; r += PZ; } else if (r >= PZ) { ++yq; r -= PZ; }
        y = yq - 1;
        z = r - 1;
        return y >= 0 && y < ny && z >= 0 && z < nz;
    };
    // rows of the B copies outside an item's gradient rows (w < 8+dz, w >= WG_ROWS+8+dz)
    // are zero in every item: written once, in every stage
    for (int e = tid; e < nst * 3 * 16 * NCG; e += WG_THREADS) {
        const int ch = e % NCG, k = (e / NCG) % 16, jz = (e / (16 * NCG)) % 3, buf = e / (3 * 16 * NCG);
        const int w = k < 7 + jz ? k : k + WG_ROWS;
        *reinterpret_cast<uint4 *>(smem + (size_t)buf * SS + BOFF + (size_t)(jz * NCG + ch) * CSB + (size_t)w * 16) =
            make_uint4(0u, 0u, 0u, 0u);
    }
    auto stage = [&](long long it, int buf) {
        const int q = (int)(it / nblk), f0 = (int)(it - (long long)q * nblk) * WG_ROWS;
        const int slo = (q / xseg) * xseg, shi = min(slo + xseg, nx);   // this sample's x-segment
        const uint32_t base = s0 + (uint32_t)buf * SS;
        // A: input planes q-1, q, q+1 (a row's grid position found once for the three)
        for (int rb = tid; rb < L; rb += WG_THREADS) {
            int y = 0, z = 0;
            const bool rv = interior(f0 - 8 - PZ + rb, y, z);
            const size_t off = ((size_t)y * nz + z) * CIN;
#pragma unroll
            for (int sp = 0; sp < 3; ++sp) {
                const int p = q - 1 + sp;
                const bool v = rv && p >= slo && p < shi;
                const __nv_bfloat16 *src = v ? in + (size_t)p * ny * nz * CIN + off : in;
                const uint32_t bytes = v ? 16u : 0u;
#pragma unroll
                for (int ch = 0; ch < NCH; ++ch)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                                 ::"r"(base + (uint32_t)(sp * NCH + ch) * CS + (uint32_t)rb * 16),
                                   "l"(src + (v ? ch * 8 : 0)), "r"(bytes));
            }
        }
        // B: gradient row f0 + r of plane q into copy dz = jz-1 at row w = r + 8 + dz
        for (int r = tid; r < WG_ROWS; r += WG_THREADS) {
            int y = 0, z = 0;
            const bool v = interior(f0 + r, y, z);
            const __nv_bfloat16 *src = v ? g + (((size_t)q * ny + y) * nz + z) * COUT : g;
            const uint32_t bytes = v ? 16u : 0u;
#pragma unroll
            for (int jz = 0; jz < 3; ++jz)
#pragma unroll
                for (int ch = 0; ch < NCG; ++ch)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                                 ::"r"(base + BOFF + (uint32_t)(jz * NCG + ch) * CSB + (uint32_t)(r + 7 + jz) * 16),
                                   "l"(src + (v ? ch * 8 : 0)), "r"(bytes));
        }
        asm volatile("cp.async.commit_group;");
    };
    // MN-major, no swizzle: 8-row K groups 128 bytes apart (LBO), 8-channel chunks CS or CSB apart (SBO)
    const uint32_t idesc = tc_idesc_n(3 * COUT) | (1u << 15) | (1u << 16);
    auto issue = [&](int buf, bool first) {
        const uint32_t base = s0 + (uint32_t)buf * SS;
        for (int kk = 0; kk < WG_K / 16; ++kk) {
            const uint64_t bd = tc_sdesc(base + BOFF + (uint32_t)(kk * 16 * 16), 128, CSB);
#pragma unroll
            for (int dyi = 0; dyi < 3; ++dyi) {
                const uint64_t ad = tc_sdesc(base + (uint32_t)((kk * 16 + dyi * PZ) * 16), 128, CS);
                const uint32_t acc = (first && kk == 0) ? 0u : 1u;
                asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                             ::"r"(tmem + (uint32_t)(dyi * 3 * COUT)), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
        }
    };

    bool ok = true;
    // nst stages: the copies of items i+1 .. i+nst-1 are in flight while item i's MMAs
    // run; one copy group per item (empty past the share) keeps the group count uniform
    for (int k = 0; k < nst - 1; ++k) {
        if (k < n_it) stage(lo + k, k);
        else asm volatile("cp.async.commit_group;");
    }
    for (long long i = 0; i < n_it; ++i) {
        const int b = (int)(i % nst);
        if (nst == 3) asm volatile("cp.async.wait_group 1;");   // item i's copies have landed
        else          asm volatile("cp.async.wait_group 0;");
        asm volatile("fence.proxy.async.shared::cta;");   // the stage is read by the tensor cores
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            issue(b, i == 0);
            tc_commit(sa(&bar_mma[b]));
        }
        // item i+nst-1 goes to the stage the previous item's MMAs read
        const long long nxt = i + nst - 1;
        if (i >= 1 && nxt < n_it &&
            !tc_wait(sa(&bar_mma[(i - 1) % nst]), (uint32_t)(((i - 1) / nst) & 1), &never))
            ok = false;
        if (ok && nxt < n_it) stage(lo + nxt, (int)(nxt % nst));
        else asm volatile("cp.async.commit_group;");
    }
    asm volatile("cp.async.wait_all;");
    __syncthreads();
    if (tid == 0 && n_it > 0) tc_commit(sa(&bar_done));   // every MMA issued above
    if (n_it > 0 && !tc_wait(sa(&bar_done), 0u, &never)) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (__syncthreads_and(ok)) {
        if (n_it > 0) {
            // lane m of the accumulators: plane q-1+s, channel ci with m = s*CIN + ci; warps
            // w and w+4 read the same lanes and share the nine accumulators
            const int m = (warp & 3) * 32 + lane;
            const int s = m / CIN, ci = m - s * CIN;
#pragma unroll 1
            for (int j = warp >> 2; j < 9; j += WG_THREADS / 128) {
                const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(j * COUT);
                uint32_t r[32];
                if (COUT == 32)
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
                                   "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
                                   "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
                                   "=r"(r[31])
                                 : "r"(taddr));
                else
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                                   "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                                 : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                if (s < 3 && ci < CINR) {
                    float *d = dW + ((size_t)(s * 9 + j) * CINR + ci) * COUTR;   // tap (dx = s-1, dy, dz)
#pragma unroll
                    for (int co = 0; co < COUTR; ++co) atomicAdd(d + co, __uint_as_float(r[co]));
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// bias gradients db[co] = sum_v g[v][co] for co < CR of C-channel rows (C divides 256)
template <typename GT>
__global__ void k_bias_grad(long long n, int C, int CR, const GT *__restrict__ g, float *db) {
    __shared__ float red[256];
    float acc = 0.f;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n * C;
         e += (long long)gridDim.x * blockDim.x) {   // a thread's channel stays threadIdx.x % C
        if constexpr (sizeof(GT) == 2) acc += __bfloat162float(g[e]); else acc += (float)g[e];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    if ((int)threadIdx.x < CR) {
        float s = 0.f;
        for (int t = threadIdx.x; t < 256; t += C) s += red[t];
        atomicAdd(&db[threadIdx.x], s);
    }
}

// per-sample squared norms of the targets: one block per sample of nsv values
__global__ void k_sample_norm(long long nsv, const float *e, float *inv_e2) {
    __shared__ double red[32 * NQ];
    const float *p = e + (long long)blockIdx.x * nsv;
    double acc[1] = {0.0};
    for (long long i = threadIdx.x; i < nsv; i += blockDim.x) acc[0] += (double)p[i] * p[i];
    block_sum<1>(acc, red);
    if (threadIdx.x == 0) inv_e2[blockIdx.x] = acc[0] > 0.0 ? (float)(1.0 / acc[0]) : 0.f;
}

// per-sample normalised squared error: L = (1/B) sum_s ||y_s - e_s||^2 / ||e_s||^2,
// g = dL/dy; samples are contiguous blocks of nsv values
__global__ void k_loss(long long n, long long nsv, int B, const float *y, const float *e, const float *inv_e2,
                       float *g, double *loss) {
    double l = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int smp = (int)(v / nsv);
        const float d = y[v] - e[v];
        const float w = inv_e2[smp] / (float)B;
        g[v] = 2.f * d * w;
        l += (double)d * d * w;
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// Adam (Kingma & Ba) on the FP32 master parameters
__global__ void k_adam(long long n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// ---- the 27-point operator on batches of crops (training loss) ---------------
// A crop is S^3 nodes with the S+1 cell planes around them; crop cell c spans
// crop nodes c-1 and c, nodes outside the crop are zero.  Per cell the edge
// differences of the node values are summed over the cell's four edges along
// each axis and weighted by the cell's hplus (the arithmetic of lap3D,
// laplacian.py:968-1015, with hplusx = hplusy = hplusz and no Coriolis or
// hcenter term); a node receives the four + side cells minus the four - side
// cells per axis, times 1/16 and 1/d^2, then diag_inv.  On nodes at least one
// node away from the crop faces this equals the full-grid operator.
__device__ __forceinline__ float crop_u(const float *u, const float *us, int S, int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= S || j >= S || k >= S) return 0.f;
    const int g = (i * S + j) * S + k;
    return us ? u[g] * us[g] : u[g];
}

__global__ void k_crop_flux(int B, int S, const float *u, const float *us, const float *h, float *F) {
    const int C = S + 1;
    const long long n = (long long)B * C * C * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(e % C);
        const long long t = e / C;
        const int d = (int)(t % C);
        const long long t2 = t / C;
        const int c = (int)(t2 % C), b = (int)(t2 / C);
        const float *ub = u + (long long)b * S * S * S;
        const float *usb = us ? us + (long long)b * S * S * S : nullptr;
        float U[2][2][2];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                for (int q = 0; q < 2; ++q) U[a][bb][q] = crop_u(ub, usb, S, c - 1 + a, d - 1 + bb, f - 1 + q);
        float xf = 0.f, yf = 0.f, zf = 0.f;
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                xf += U[1][p][q] - U[0][p][q];
                yf += U[p][1][q] - U[p][0][q];
                zf += U[p][q][1] - U[p][q][0];
            }
        const float hh = h[e];
        F[3 * e + 0] = hh * xf;
        F[3 * e + 1] = hh * yf;
        F[3 * e + 2] = hh * zf;
    }
}

// out = dinv * (node sums of F), zero on nodes within `margin` nodes of the crop's faces
__global__ void k_crop_node(int B, int S, const float *F, const float *dinv, float ox, float oy, float oz,
                            int margin, float *out) {
    const int C = S + 1;
    const long long n = (long long)B * S * S * S;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e % S);
        const long long t = e / S;
        const int j = (int)(t % S);
        const long long t2 = t / S;
        const int i = (int)(t2 % S), b = (int)(t2 / S);
        const float *Fb = F + (long long)b * C * C * C * 3;
        auto at = [&](int c, int d, int f, int comp) { return Fb[(((long long)c * C + d) * C + f) * 3 + comp]; };
        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                sx += at(i + 1, j + p, k + q, 0) - at(i, j + p, k + q, 0);
                sy += at(i + p, j + 1, k + q, 1) - at(i + p, j, k + q, 1);
                sz += at(i + p, j + q, k + 1, 2) - at(i + p, j + q, k, 2);
            }
        float v = 0.0625f * (ox * sx + oy * sy + oz * sz);
        if (dinv) v *= dinv[e];
        if (i < margin || j < margin || k < margin || i >= S - margin || j >= S - margin || k >= S - margin) v = 0.f;
        out[e] = v;
    }
}

// d = a - b (node grid)
__global__ void k_sub(long long n, const float *a, const float *b, float *d) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = a[i] - b[i];
}

// per-sample weights 1/||core(r_s)||^2 (one block per sample; core: nodes at least
// `margin` nodes inside the crop)
__global__ void k_crop_rnorm(int S, int margin, const float *r, double *acc) {
    // one block per (x-plane of the core, sample): partial sums of r^2 over the core
    __shared__ double red[32 * NQ];
    const int W = S - 2 * margin;
    const float *p = r + ((long long)blockIdx.y * S + margin + blockIdx.x) * S * S;
    double a[1] = {0.0};
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        const int jj = e / W;
        const float v = p[(margin + jj) * S + margin + (e - jj * W)];
        a[0] += (double)v * v;
    }
    block_sum<1>(a, red);
    if (threadIdx.x == 0) atomicAdd(&acc[blockIdx.y], a[0]);
}

// w_s = 1 / sum over the core of r^2 (0 for an all-zero core)
__global__ void k_crop_rinv(int B, const double *acc, float *w) {
    const int smp = blockIdx.x * blockDim.x + threadIdx.x;
    if (smp < B) w[smp] = acc[smp] > 0.0 ? (float)(1.0 / acc[smp]) : 0.f;
}

// loss += w_s ||q||^2 / B and q *= 2 w_s / B (q becomes dL/d(Ad) before the adjoint)
__global__ void k_crop_loss(long long n, long long nsv, int B, float *q, const float *w, double *loss) {
    double l = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float ws = w[v / nsv] / (float)B;
        const float qv = q[v];
        l += (double)qv * qv * ws;
        q[v] = 2.f * ws * qv;
    }
    l = warp_sum(l);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

}  // namespace bella

// ============================================================================
// C ABI
// ============================================================================
using namespace bella;

// Layer shapes: real channels (cin, cout) and the padded kernel shapes (cinp, coutp);
// layer 0 takes block^3 sub-node channels (padded to 16), layer 5 returns block^3
// channels (padded to 8; to 16 for its mirrored input-gradient pass).
struct bella_cnn {
    int device, block;
    int linear;               // 1: no ReLU and no biases (a linear map)
    int use_tc;               // 1: the forward pass on tcgen05 (k_conv3d_tc)
    __nv_bfloat16 *wtc[6];    // its weights in tensor-core operand order (layer 5: 16 output rows)
    __nv_bfloat16 *wtcT[6];   // layers 1-5: the input-gradient pass's weights in that order
    int *tc_err;              // set when a tensor-core wait gave up
    float omega;              // identity path: output = omega * input + network
    int bias_free;            // 1: biases held at zero (positively homogeneous map)
    long long cap;            // net-grid voxel capacity
    int cin[6], cout[6];
    float *params, *grads, *adam_m, *adam_v;   // FP32, layout W[l][27][cin][cout], b[l][cout]
    long long nparams;
    long long adam_t;
    __nv_bfloat16 *wk[6], *wkT[6];   // [27][coutp][cinp] and mirrored [27][cinp][coutpT]
    float *bias[6];
    __nv_bfloat16 *act[6];    // act[0]: packed input (16 ch); act[l]: output of layer l-1 (32 ch)
    __nv_bfloat16 *gact[2];   // gradient ping-pong (32 ch; gact[1] also holds the 16-ch output gradient)
    float *y8, *t8, *g8;      // net output, target, output gradient [cap][8]
    float *inv_e2;            // per-sample 1/||target||^2 [cap]
    double *loss;
    // operator-loss scratch (node grid of a batch of crops), allocated on first use
    float *yf, *qf, *gf, *flux, *wcrop;   // wcrop: per-sample loss weights, then their FP64 sums
    long long fine_cap, flux_cap;
    long long launches;
};

static const int CINP_L[6] = {16, 32, 32, 32, 32, 32};
static const int COUTP_L[6] = {32, 32, 32, 32, 32, 8};
static const int COUTPT_L[6] = {32, 32, 32, 32, 32, 16};
static const int COUTTC_L[6] = {32, 32, 32, 32, 32, 16};   // tensor-core B rows per dx tap

static long long param_count_b(int block) {
    const int b3 = block * block * block;
    const int cin[6] = {b3, 32, 32, 32, 32, 32}, cout[6] = {32, 32, 32, 32, 32, b3};
    long long n = 0;
    for (int l = 0; l < 6; ++l) n += 27LL * cin[l] * cout[l] + cout[l];
    return n;
}

static long long w_off(const bella_cnn *net, int l) {
    long long n = 0;
    for (int k = 0; k < l; ++k) n += 27LL * net->cin[k] * net->cout[k] + net->cout[k];
    return n;
}

// master f32 [27][cin][cout] -> kernel bf16 [27][coutp][cinp] and the mirrored
// transpose [27][cinp][coutpT] used by the input-gradient pass
__global__ void k_cast_weights(const float *W, int cin, int cout, int cinp, int coutp, int coutpT,
                               __nv_bfloat16 *wk, __nv_bfloat16 *wkT) {
    const int total = 27 * cinp * coutpT;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int tap = e / (cinp * coutpT), r = e - tap * cinp * coutpT, co = r / cinp, ci = r - co * cinp;
        float v = 0.f;
        if (ci < cin && co < cout) v = W[((size_t)tap * cin + ci) * cout + co];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        if (co < coutp) wk[((size_t)tap * coutp + co) * cinp + ci] = h;
        wkT[((size_t)tap * cinp + ci) * coutpT + co] = h;
    }
}

__global__ void k_cast_bias(const float *b, int cout, int coutp, float *bp) {
    for (int e = threadIdx.x; e < coutp; e += blockDim.x) bp[e] = e < cout ? b[e] : 0.f;
}

static void cnn_free(bella_cnn *net) {
    cudaFree(net->params); cudaFree(net->grads); cudaFree(net->adam_m); cudaFree(net->adam_v);
    for (int l = 0; l < 6; ++l) { cudaFree(net->wk[l]); cudaFree(net->wkT[l]); cudaFree(net->bias[l]); cudaFree(net->act[l]); }
    cudaFree(net->gact[0]); cudaFree(net->gact[1]);
    cudaFree(net->y8); cudaFree(net->t8); cudaFree(net->g8); cudaFree(net->inv_e2); cudaFree(net->loss);
    cudaFree(net->yf); cudaFree(net->qf); cudaFree(net->gf); cudaFree(net->flux); cudaFree(net->wcrop);
    for (int l = 0; l < 6; ++l) { cudaFree(net->wtc[l]); cudaFree(net->wtcT[l]); }
    cudaFree(net->tc_err);
}

template <typename K>
static bool big_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess;
}

static int conv_grid(const BlockMap &m) {
    const long long tiles = (long long)m.B * ((m.cx + CT_X - 1) / CT_X) * ((m.cy + CT_Y - 1) / CT_Y) *
                            ((m.cz + CT_Z - 1) / CT_Z);
    const long long cap = (long long)num_sms() * 2;
    return (int)(tiles < cap ? tiles : cap);
}

// the conv kernels see the stacked samples as one (B*cx, cy, cz) grid cut into
// x segments of cx voxels; B > 1 needs cx to be a multiple of the tile width
static bool map_ok(const bella_cnn *net, const BlockMap &m) {
    return m.nvox() <= net->cap && (m.B == 1 || m.cx % CT_X == 0);
}

// a launch that may begin while the previous kernel in the stream is finishing
// (programmatic dependent launch); the kernel orders itself with griddepcontrol.wait
template <typename... P, typename... A>
static void launch_dependent(void (*kernel)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<P>(args)...);
}

static int tc_grid(long long nitems) {
    int nsm = num_sms();
    return (int)(nitems < nsm ? nitems : nsm);
}

// the forward pass on tcgen05 when enabled and the staged planes fit in shared memory
static bool tc_fits(const BlockMap &m) {
    return tc_smem_bytes<32, 32>(m.cz + 2) <= TC_SMEM_MAX;
}

static void forward_layers(bella_cnn *net, const BlockMap &m, float out_scale, cudaStream_t s) {
    const int g = conv_grid(m);
    const int nx = m.B * m.cx, ny = m.cy, nz = m.cz, xs = m.cx;
    if (net->use_tc && tc_fits(m)) {
        // the (row block, x-plane) items shared evenly, one CTA per SM
        const long long plane = (long long)(ny + 2) * (nz + 2);
        const long long items = ((plane + TC_ROWS - 1) / TC_ROWS) * (long long)nx;
        const int gt = tc_grid(items), pz = nz + 2;
        const long long work = (items + gt - 1) / gt;
        const float *b5 = net->linear ? nullptr : net->bias[5];
        // layers 2..6 are programmatic dependents of the layer before (one CTA per SM
        // each, so the whole previous grid is resident when they launch)
        const __nv_bfloat16 *nomask = nullptr;
        if (net->linear) {
            k_conv3d_tc<16, 32, false, false><<<gt, TC_THREADS, tc_smem_bytes<16, 32>(pz), s>>>(
                nx, ny, nz, xs, work, net->act[0], net->wtc[0], nullptr, net->act[1], 1.f, net->tc_err, nullptr);
            for (int l = 1; l <= 4; ++l)
                launch_dependent(k_conv3d_tc<32, 32, false, false>, gt, TC_THREADS, tc_smem_bytes<32, 32>(pz), s,
                                 nx, ny, nz, xs, work, net->act[l], net->wtc[l], (const float *)nullptr,
                                 (void *)net->act[l + 1], 1.f, net->tc_err, nomask);
        } else {
            k_conv3d_tc<16, 32, true, false><<<gt, TC_THREADS, tc_smem_bytes<16, 32>(pz), s>>>(
                nx, ny, nz, xs, work, net->act[0], net->wtc[0], net->bias[0], net->act[1], 1.f, net->tc_err, nullptr);
            for (int l = 1; l <= 4; ++l)
                launch_dependent(k_conv3d_tc<32, 32, true, false>, gt, TC_THREADS, tc_smem_bytes<32, 32>(pz), s,
                                 nx, ny, nz, xs, work, net->act[l], net->wtc[l], (const float *)net->bias[l],
                                 (void *)net->act[l + 1], 1.f, net->tc_err, nomask);
        }
        launch_dependent(k_conv3d_tc<32, 16, false, true>, gt, TC_THREADS, tc_smem_bytes<32, 16>(pz), s,
                         nx, ny, nz, xs, work, net->act[5], net->wtc[5], b5, (void *)net->y8, out_scale,
                         net->tc_err, nomask);
        net->launches += 6;
        return;
    }
    if (net->linear) {
        k_conv3d<16, 32, false, false, false><<<g, CNN_THREADS, conv_smem<16, 32>(), s>>>(
            nx, ny, nz, xs, net->act[0], net->wk[0], nullptr, net->act[1], 1.f, nullptr);
        for (int l = 1; l <= 4; ++l)
            k_conv3d<32, 32, false, false, false><<<g, CNN_THREADS, conv_smem<32, 32>(), s>>>(
                nx, ny, nz, xs, net->act[l], net->wk[l], nullptr, net->act[l + 1], 1.f, nullptr);
        k_conv3d<32, 8, false, true, false><<<g, CNN_THREADS, conv_smem<32, 8>(), s>>>(
            nx, ny, nz, xs, net->act[5], net->wk[5], nullptr, net->y8, out_scale, nullptr);
    } else {
        k_conv3d<16, 32, true, false, false><<<g, CNN_THREADS, conv_smem<16, 32>(), s>>>(
            nx, ny, nz, xs, net->act[0], net->wk[0], net->bias[0], net->act[1], 1.f, nullptr);
        for (int l = 1; l <= 4; ++l)
            k_conv3d<32, 32, true, false, false><<<g, CNN_THREADS, conv_smem<32, 32>(), s>>>(
                nx, ny, nz, xs, net->act[l], net->wk[l], net->bias[l], net->act[l + 1], 1.f, nullptr);
        k_conv3d<32, 8, false, true, false><<<g, CNN_THREADS, conv_smem<32, 8>(), s>>>(
            nx, ny, nz, xs, net->act[5], net->wk[5], net->bias[5], net->y8, out_scale, nullptr);
    }
    net->launches += 6;
}

// gradients of sum(g8 * y8) into net->grads (zeroed here), from the stored activations
static void backward_layers(bella_cnn *net, const BlockMap &m, cudaStream_t s) {
    const int g = conv_grid(m);
    const int nx = m.B * m.cx, ny = m.cy, nz = m.cz, xs = m.cx;
    const long long n = m.nvox();
    const int gw = g < num_sms() ? g : num_sms();
    cudaMemsetAsync(net->grads, 0, net->nparams * sizeof(float), s);
    float *dW[6], *db[6];
    for (int l = 0; l < 6; ++l) {
        dW[l] = net->grads + w_off(net, l);
        db[l] = dW[l] + 27LL * net->cin[l] * net->cout[l];
    }
    // the tcgen05 kernels (input gradients: the forward kernel with the mirrored,
    // transposed weights and, with ReLUs, the ReLU derivative in its epilogue; weight
    // gradients: k_wgrad_tc) where the staged planes fit, else mma.sync and FP32 loops
    const bool relu = !net->linear;
    const bool tc = net->use_tc && tc_fits(m);
    const bool wtc = net->use_tc && 2 * (size_t)wg_stage_bytes(32, 32, nz + 2) <= TC_SMEM_MAX;
    const bool bias = !(net->linear || net->bias_free);
    const long long plane = (long long)(ny + 2) * (nz + 2);
    const long long items = ((plane + TC_ROWS - 1) / TC_ROWS) * (long long)nx;
    const int gt = tc_grid(items), pz = nz + 2;
    const long long work = (items + gt - 1) / gt;
    const long long witems = ((plane + WG_ROWS - 1) / WG_ROWS) * (long long)nx;
    const int gwt = tc_grid(witems);
    const long long wwork = (witems + gwt - 1) / gwt;
    const int gb = vec_grid(n);
    long long launches = 0;
    // layer 5 (32 -> block^3)
    if (wtc) {
        k_g8_to_bf16<<<vec_grid(n), 256, 0, s>>>(n, net->g8, net->gact[1]);
        if (net->block == 2)
            k_wgrad_tc<32, 16, 32, 8><<<gwt, WG_THREADS, wg_smem_bytes(32, 16, pz), s>>>(
                nx, ny, nz, xs, wwork, wg_stages(32, 16, pz), net->act[5], net->gact[1], dW[5], net->tc_err);
        else
            k_wgrad_tc<32, 16, 32, 1><<<gwt, WG_THREADS, wg_smem_bytes(32, 16, pz), s>>>(
                nx, ny, nz, xs, wwork, wg_stages(32, 16, pz), net->act[5], net->gact[1], dW[5], net->tc_err);
        if (bias) k_bias_grad<float><<<gb, 256, 0, s>>>(n, 8, net->block == 2 ? 8 : 1, net->g8, db[5]);
        launches += 2 + (bias ? 1 : 0);
    } else {
        if (net->block == 2)
            k_wgrad<32, 32, 8, 8, float><<<gw, 256, wgrad_smem<32, 8>(), s>>>(nx, ny, nz, xs, net->act[5], net->g8,
                                                                              dW[5], db[5]);
        else
            k_wgrad<32, 32, 8, 1, float><<<gw, 256, wgrad_smem<32, 1>(), s>>>(nx, ny, nz, xs, net->act[5], net->g8,
                                                                              dW[5], db[5]);
        k_g8_to_bf16<<<vec_grid(n), 256, 0, s>>>(n, net->g8, net->gact[1]);
        launches += 2;
    }
    if (tc)
        k_conv3d_tc<16, 32, false, false><<<gt, TC_THREADS, tc_smem_bytes<16, 32>(pz), s>>>(
            nx, ny, nz, xs, work, net->gact[1], net->wtcT[5], nullptr, net->gact[0], 1.f, net->tc_err,
            relu ? net->act[5] : nullptr);
    else
        k_conv3d<16, 32, false, false, true><<<g, CNN_THREADS, conv_smem<16, 32>(), s>>>(
            nx, ny, nz, xs, net->gact[1], net->wkT[5], nullptr, net->gact[0], 1.f, relu ? net->act[5] : nullptr);
    launches += 1;
    int cur = 0;
    for (int l = 4; l >= 1; --l) {
        if (wtc) {
            k_wgrad_tc<32, 32, 32, 32><<<gwt, WG_THREADS, wg_smem_bytes(32, 32, pz), s>>>(
                nx, ny, nz, xs, wwork, wg_stages(32, 32, pz), net->act[l], net->gact[cur], dW[l], net->tc_err);
            if (bias) k_bias_grad<__nv_bfloat16><<<gb, 256, 0, s>>>(n, 32, 32, net->gact[cur], db[l]);
            launches += 1 + (bias ? 1 : 0);
        } else {
            k_wgrad<32, 32, 32, 32, __nv_bfloat16><<<gw, 256, wgrad_smem<32, 32>(), s>>>(
                nx, ny, nz, xs, net->act[l], net->gact[cur], dW[l], db[l]);
            launches += 1;
        }
        if (tc)
            k_conv3d_tc<32, 32, false, false><<<gt, TC_THREADS, tc_smem_bytes<32, 32>(pz), s>>>(
                nx, ny, nz, xs, work, net->gact[cur], net->wtcT[l], nullptr, net->gact[cur ^ 1], 1.f, net->tc_err,
                relu ? net->act[l] : nullptr);
        else
            k_conv3d<32, 32, false, false, true><<<g, CNN_THREADS, conv_smem<32, 32>(), s>>>(
                nx, ny, nz, xs, net->gact[cur], net->wkT[l], nullptr, net->gact[cur ^ 1], 1.f,
                relu ? net->act[l] : nullptr);
        launches += 1;
        cur ^= 1;
    }
    if (wtc) {
        if (net->block == 2)
            k_wgrad_tc<16, 32, 8, 32><<<gwt, WG_THREADS, wg_smem_bytes(16, 32, pz), s>>>(
                nx, ny, nz, xs, wwork, wg_stages(16, 32, pz), net->act[0], net->gact[cur], dW[0], net->tc_err);
        else
            k_wgrad_tc<16, 32, 1, 32><<<gwt, WG_THREADS, wg_smem_bytes(16, 32, pz), s>>>(
                nx, ny, nz, xs, wwork, wg_stages(16, 32, pz), net->act[0], net->gact[cur], dW[0], net->tc_err);
        if (bias) k_bias_grad<__nv_bfloat16><<<gb, 256, 0, s>>>(n, 32, 32, net->gact[cur], db[0]);
        launches += 1 + (bias ? 1 : 0);
    } else {
        if (net->block == 2)
            k_wgrad<16, 8, 32, 32, __nv_bfloat16><<<gw, 256, wgrad_smem<8, 32>(), s>>>(
                nx, ny, nz, xs, net->act[0], net->gact[cur], dW[0], db[0]);
        else
            k_wgrad<16, 1, 32, 32, __nv_bfloat16><<<gw, 256, wgrad_smem<1, 32>(), s>>>(
                nx, ny, nz, xs, net->act[0], net->gact[cur], dW[0], db[0]);
        launches += 1;
    }
    net->launches += launches;
    if (!bias) {   // biases stay at zero: no gradient, no Adam motion
        for (int l = 0; l < 6; ++l) cudaMemsetAsync(db[l], 0, net->cout[l] * sizeof(float), s);
    }
}

// refresh the BF16 kernel weights from the FP32 master parameters (device)
static int cnn_sync_weights(bella_cnn *net, cudaStream_t s) {
    for (int l = 0; l < 6; ++l) {
        const float *W = net->params + w_off(net, l);
        const float *b = W + 27LL * net->cin[l] * net->cout[l];
        k_cast_weights<<<64, 256, 0, s>>>(W, net->cin[l], net->cout[l], CINP_L[l], COUTP_L[l], COUTPT_L[l],
                                          net->wk[l], net->wkT[l]);
        k_cast_bias<<<1, 32, 0, s>>>(b, net->cout[l], COUTP_L[l], net->bias[l]);
        net->launches += 2;
        if (net->wtc[l]) {
            k_wk_to_tc<<<64, 256, 0, s>>>(net->wk[l], CINP_L[l], COUTP_L[l], COUTTC_L[l], net->wtc[l], 0);
            net->launches += 1;
        }
        if (l >= 1 && net->wtcT[l]) {   // the input-gradient pass of layer l: mirrored taps, (ci, co) swapped
            k_wk_to_tc<<<64, 256, 0, s>>>(net->wkT[l], COUTPT_L[l], CINP_L[l], CINP_L[l], net->wtcT[l], 1);
            net->launches += 1;
        }
    }
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

static std::string g_cnn_err;

namespace bella {
// out = CNN(in / rms) * rms with rms = sqrt(*sumsq / n) read on the device (no host
// synchronisation); used by the flexible solver.  BELLA_EINVAL if the grid
// exceeds the network's capacity.
int cnn_apply_dev(bella_cnn *net, int nx, int ny, int nz, const float *in, float *out, const double *sumsq,
                  cudaStream_t s, const int *per) {
    const BlockMap m = make_map(1, nx, ny, nz, net->block);
    if (!map_ok(net, m)) return BELLA_EINVAL;
    pack_in(m, in, 1.f, net->act[0], sumsq, s);
    forward_layers(net, m, 1.f, s);
    const int pmask = per ? (per[0] ? 1 : 0) | (per[1] ? 2 : 0) | (per[2] ? 4 : 0) : 0;
    const int seam = 7 * net->block - 1;      // six 3x3x3 layers on b-node blocks: 6b + (b - 1) nodes
    unpack(m, net->y8, out, sumsq, in, net->omega, pmask, seam, s);
    net->launches += 2;
    return BELLA_OK;
}
}  // namespace bella

extern "C" {

int bella_cnn_create(bella_cnn **out, int device, int block, long long capacity) {
    if (!out || capacity <= 0 || (block != 1 && block != 2)) return BELLA_EINVAL;
    if (capacity * 8 >= (1LL << 31)) return BELLA_EINVAL;   // the pack kernels index nodes in 32 bits
    if (cudaSetDevice(device) != cudaSuccess) return BELLA_ECUDA;
    bella_cnn *net = new bella_cnn();
    memset(net, 0, sizeof(*net));
    net->device = device;
    net->block = block;
    net->cap = capacity;
    const int b3 = block * block * block;
    for (int l = 0; l < 6; ++l) { net->cin[l] = l == 0 ? b3 : 32; net->cout[l] = l == 5 ? b3 : 32; }
    net->nparams = param_count_b(block);
    net->use_tc = 1;                 // tcgen05 forward where the staged planes fit (mma.sync otherwise)
    const size_t C = (size_t)capacity;
    bool ok = true;
    for (float **p : {&net->params, &net->grads, &net->adam_m, &net->adam_v})
        ok = ok && cudaMalloc(p, net->nparams * sizeof(float)) == cudaSuccess;
    for (int l = 0; l < 6 && ok; ++l) {
        ok = cudaMalloc(&net->wk[l], 27ULL * CINP_L[l] * COUTP_L[l] * 2) == cudaSuccess &&
             cudaMalloc(&net->wkT[l], 27ULL * CINP_L[l] * COUTPT_L[l] * 2) == cudaSuccess &&
             cudaMalloc(&net->bias[l], 32 * sizeof(float)) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&net->act[0], C * 16 * 2) == cudaSuccess;
    for (int l = 1; l < 6 && ok; ++l) ok = cudaMalloc(&net->act[l], C * 32 * 2) == cudaSuccess;
    for (int k = 0; k < 2 && ok; ++k) ok = cudaMalloc(&net->gact[k], C * 32 * 2) == cudaSuccess;
    for (float **p : {&net->y8, &net->t8, &net->g8}) ok = ok && cudaMalloc(p, C * 8 * sizeof(float)) == cudaSuccess;
    ok = ok && cudaMalloc(&net->inv_e2, C * sizeof(float)) == cudaSuccess;
    for (int l = 0; l < 6 && ok; ++l) ok = cudaMalloc(&net->wtc[l], 27ULL * CINP_L[l] * COUTTC_L[l] * 2) == cudaSuccess;
    for (int l = 1; l < 6 && ok; ++l) ok = cudaMalloc(&net->wtcT[l], 27ULL * COUTPT_L[l] * CINP_L[l] * 2) == cudaSuccess;
    ok = ok && cudaMalloc(&net->tc_err, sizeof(int)) == cudaSuccess && cudaMemset(net->tc_err, 0, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMalloc(&net->loss, sizeof(double)) == cudaSuccess;
    for (float *p : {net->params, net->grads, net->adam_m, net->adam_v})
        ok = ok && cudaMemset(p, 0, net->nparams * sizeof(float)) == cudaSuccess;
    ok = ok && big_smem(k_conv3d<16, 32, true, false, false>, conv_smem<16, 32>()) &&
         big_smem(k_conv3d<32, 32, true, false, false>, conv_smem<32, 32>()) &&
         big_smem(k_conv3d<32, 8, false, true, false>, conv_smem<32, 8>()) &&
         big_smem(k_conv3d<32, 32, false, false, true>, conv_smem<32, 32>()) &&
         big_smem(k_conv3d<16, 32, false, false, true>, conv_smem<16, 32>()) &&
         big_smem(k_conv3d<16, 32, false, false, false>, conv_smem<16, 32>()) &&
         big_smem(k_conv3d<32, 32, false, false, false>, conv_smem<32, 32>()) &&
         big_smem(k_wgrad<32, 32, 8, 8, float>, wgrad_smem<32, 8>()) &&
         big_smem(k_wgrad<32, 32, 8, 1, float>, wgrad_smem<32, 1>()) &&
         big_smem(k_wgrad<32, 32, 32, 32, __nv_bfloat16>, wgrad_smem<32, 32>()) &&
         big_smem(k_wgrad<16, 8, 32, 32, __nv_bfloat16>, wgrad_smem<8, 32>()) &&
         big_smem(k_wgrad<16, 1, 32, 32, __nv_bfloat16>, wgrad_smem<1, 32>()) &&
         big_smem(k_conv3d_tc<16, 32, false, false>, TC_SMEM_MAX) &&
         big_smem(k_conv3d_tc<16, 32, true, false>, TC_SMEM_MAX) &&
         big_smem(k_conv3d_tc<32, 32, false, false>, TC_SMEM_MAX) &&
         big_smem(k_conv3d_tc<32, 32, true, false>, TC_SMEM_MAX) && big_smem(k_conv3d_tc<32, 16, false, true>, TC_SMEM_MAX) &&
         big_smem(k_wgrad_tc<32, 16, 32, 8>, TC_SMEM_MAX) && big_smem(k_wgrad_tc<32, 16, 32, 1>, TC_SMEM_MAX) &&
         big_smem(k_wgrad_tc<32, 32, 32, 32>, TC_SMEM_MAX) && big_smem(k_wgrad_tc<16, 32, 8, 32>, TC_SMEM_MAX) &&
         big_smem(k_wgrad_tc<16, 32, 1, 32>, TC_SMEM_MAX);
    if (ok) ok = cnn_sync_weights(net, 0) == BELLA_OK && cudaDeviceSynchronize() == cudaSuccess;
    if (!ok) {
        g_cnn_err = "bella_cnn_create: allocation or attribute failed";
        cnn_free(net);
        delete net;
        return BELLA_ECUDA;
    }
    *out = net;
    return BELLA_OK;
}

int bella_cnn_destroy(bella_cnn *net) {
    if (!net) return BELLA_OK;
    cudaSetDevice(net->device);
    cnn_free(net);
    delete net;
    return BELLA_OK;
}

long long bella_cnn_param_count(int block) { return (block == 1 || block == 2) ? param_count_b(block) : -1; }

// params: host or device FP32 array of bella_cnn_param_count(block) values, layer
// by layer W[27][cin][cout] then b[cout].  Resets the Adam state.
int bella_cnn_set_params(bella_cnn *net, const float *params, void *stream) {
    if (!net || !params) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(net->params, params, net->nparams * sizeof(float), cudaMemcpyDefault, s) != cudaSuccess)
        return BELLA_ECUDA;
    cudaMemsetAsync(net->adam_m, 0, net->nparams * sizeof(float), s);
    cudaMemsetAsync(net->adam_v, 0, net->nparams * sizeof(float), s);
    net->adam_t = 0;
    return cnn_sync_weights(net, s);
}

int bella_cnn_get_params(bella_cnn *net, float *params, void *stream) {
    if (!net || !params) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(params, net->params, net->nparams * sizeof(float), cudaMemcpyDefault, s) != cudaSuccess)
        return BELLA_ECUDA;
    return BELLA_OK;
}

// out = CNN(in * in_scale) / in_scale on the nodes of an (nx, ny, nz) grid (C
// order, z fastest); in and out are device FP32 arrays and may not alias
int bella_cnn_forward(bella_cnn *net, int nx, int ny, int nz, const float *in, float *out, float in_scale,
                      void *stream) {
    if (!net || !in || !out || nx < 1 || ny < 1 || nz < 1 || !(in_scale > 0.f)) return BELLA_EINVAL;
    const BlockMap m = make_map(1, nx, ny, nz, net->block);
    if (!map_ok(net, m)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    pack_in(m, in, in_scale, net->act[0], nullptr, s);
    forward_layers(net, m, 1.f / in_scale, s);
    unpack(m, net->y8, out, nullptr, in, net->omega, 0, 0, s);
    net->launches += 2;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// Parameter gradients of sum(gout * CNN(in)) (nodes of an (nx, ny, nz) grid,
// device FP32) into grads (device FP32, parameter layout).  Also leaves the
// forward output in `out` when non-null.
int bella_cnn_gradients(bella_cnn *net, int nx, int ny, int nz, const float *in, const float *gout, float *grads,
                        float *out, void *stream) {
    if (!net || !in || !gout || !grads || nx < 1 || ny < 1 || nz < 1) return BELLA_EINVAL;
    const BlockMap m = make_map(1, nx, ny, nz, net->block);
    if (!map_ok(net, m)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    pack_in(m, in, 1.f, net->act[0], nullptr, s);
    forward_layers(net, m, 1.f, s);
    if (out) unpack(m, net->y8, out, nullptr, in, net->omega, 0, 0, s);
    k_pack_f32<<<vec_grid(m.nvox()), 256, 0, s>>>(m, gout, 1.f, net->g8);
    backward_layers(net, m, s);
    cudaMemcpyAsync(grads, net->grads, net->nparams * sizeof(float), cudaMemcpyDeviceToDevice, s);
    net->launches += 3;
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// One Adam step on a batch of nsamples (input, target) pairs of (nx, ny, nz)
// nodes each, stacked as [nsamples][nx][ny][nz] device FP32 arrays.  The loss
// is the mean over samples of ||CNN(in_s) - target_s||^2 / ||target_s||^2; the
// caller normalises each pair (the solver feeds the net unit-RMS inputs).
// nx, ny, nz must be multiples of the block size and, for nsamples > 1,
// nx / block a multiple of 4.  *loss (host, optional) receives the batch loss
// before the step, which synchronises the stream.
int bella_cnn_train_step(bella_cnn *net, int nsamples, int nx, int ny, int nz, const float *in, const float *target,
                         float lr, double *loss, void *stream) {
    if (!net || !in || !target || nsamples < 1 || nx < 1 || ny < 1 || nz < 1 || !(lr > 0.f)) return BELLA_EINVAL;
    const int b = net->block;
    if (nx % b || ny % b || nz % b) return BELLA_EINVAL;
    const BlockMap m = make_map(nsamples, nx, ny, nz, b);
    if (!map_ok(net, m)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = m.nvox();
    const long long nsv = (long long)m.cx * m.cy * m.cz * 8;
    pack_in(m, in, 1.f, net->act[0], nullptr, s);
    k_pack_f32<<<vec_grid(n), 256, 0, s>>>(m, target, 1.f, net->t8);
    k_sample_norm<<<nsamples, 256, 0, s>>>(nsv, net->t8, net->inv_e2);
    forward_layers(net, m, 1.f, s);
    cudaMemsetAsync(net->loss, 0, sizeof(double), s);
    k_loss<<<vec_grid(n * 8), 256, 0, s>>>(n * 8, nsv, nsamples, net->y8, net->t8, net->inv_e2, net->g8, net->loss);
    backward_layers(net, m, s);
    net->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - powf(b1, (float)net->adam_t), bc2 = 1.f - powf(b2, (float)net->adam_t);
    k_adam<<<vec_grid(net->nparams), 256, 0, s>>>(net->nparams, net->params, net->grads, net->adam_m, net->adam_v, lr,
                                                  b1, b2, 1e-8f, bc1, bc2);
    net->launches += 5;
    const int rc = cnn_sync_weights(net, s);
    if (rc != BELLA_OK) return rc;
    if (loss) {
        if (cudaMemcpyAsync(loss, net->loss, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return BELLA_ECUDA;
    }
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// y = A_crop u for nsamples crops of S^3 nodes (device FP32): hcell
// [nsamples][(S+1)^3] cell hplus, dinv [nsamples][S^3]; y is zero on nodes
// within `margin` nodes of the crop's faces.  Scratch flux: [nsamples][(S+1)^3][3].
int bella_crop_apply(int nsamples, int S, const float *u, const float *hcell, const float *dinv, double dx, double dy,
                     double dz, int margin, float *flux, float *y, void *stream) {
    if (nsamples < 1 || S < 2 || margin < 0 || !u || !hcell || !flux || !y) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    const long long nc = (long long)nsamples * (S + 1) * (S + 1) * (S + 1), nn = (long long)nsamples * S * S * S;
    k_crop_flux<<<vec_grid(nc), 256, 0, s>>>(nsamples, S, u, nullptr, hcell, flux);
    k_crop_node<<<vec_grid(nn), 256, 0, s>>>(nsamples, S, flux, dinv, (float)(1.0 / (dx * dx)),
                                             (float)(1.0 / (dy * dy)), (float)(1.0 / (dz * dz)), margin, y);
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

// One Adam step on the operator residual of the predicted error:
//   loss = mean_s ||core(A_s (M(r_s) - e_s))||^2 / ||core(r_s)||^2
// for nsamples crops of S^3 nodes, M the map with its identity path, core the
// nodes at least `margin` nodes inside the crop (r = A e on the full grid, so
// there A(M(r) - e) = A M(r) - r).  A margin of the network's reach plus one
// keeps the loss where the network never sees the crop's zero padding, as in
// the bulk of a solve.  hcell, dinv: the crops' operator coefficients as in
// bella_crop_apply; the gradient through A uses A^T = L diag(dinv) with L the
// symmetric unscaled operator.
int bella_cnn_train_step_op(bella_cnn *net, int nsamples, int S, const float *in, const float *target,
                            const float *hcell, const float *dinv, double dx, double dy, double dz, int margin,
                            float lr, double *loss, void *stream) {
    if (!net || !in || !target || !hcell || !dinv || nsamples < 1 || S < 4 || margin < 1 || 2 * margin >= S ||
        !(lr > 0.f))
        return BELLA_EINVAL;
    const int b = net->block;
    if (S % b) return BELLA_EINVAL;
    const BlockMap m = make_map(nsamples, S, S, S, b);
    if (!map_ok(net, m)) return BELLA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    const long long nn = (long long)nsamples * S * S * S;
    const long long nc = (long long)nsamples * (S + 1) * (S + 1) * (S + 1);
    if (net->fine_cap < nn) {
        cudaFree(net->yf); cudaFree(net->qf); cudaFree(net->gf); cudaFree(net->wcrop);
        net->yf = net->qf = net->gf = net->wcrop = nullptr;
        net->fine_cap = 0;
        if (cudaMalloc(&net->yf, nn * 4) != cudaSuccess || cudaMalloc(&net->qf, nn * 4) != cudaSuccess ||
            cudaMalloc(&net->gf, nn * 4) != cudaSuccess || cudaMalloc(&net->wcrop, (nn / 64 + 1) * 16) != cudaSuccess)
            return BELLA_ECUDA;
        net->fine_cap = nn;
    }
    if (net->flux_cap < nc) {
        cudaFree(net->flux);
        net->flux = nullptr;
        net->flux_cap = 0;
        if (cudaMalloc(&net->flux, nc * 3 * 4) != cudaSuccess) return BELLA_ECUDA;
        net->flux_cap = nc;
    }
    const float ox = (float)(1.0 / (dx * dx)), oy = (float)(1.0 / (dy * dy)), oz = (float)(1.0 / (dz * dz));
    pack_in(m, in, 1.f, net->act[0], nullptr, s);
    forward_layers(net, m, 1.f, s);
    unpack(m, net->y8, net->yf, nullptr, in, net->omega, 0, 0, s);
    k_sub<<<vec_grid(nn), 256, 0, s>>>(nn, net->yf, target, net->gf);
    // q = interior(A (y - e))
    k_crop_flux<<<vec_grid(nc), 256, 0, s>>>(nsamples, S, net->gf, nullptr, hcell, net->flux);
    k_crop_node<<<vec_grid(nn), 256, 0, s>>>(nsamples, S, net->flux, dinv, ox, oy, oz, margin, net->qf);
    double *rsum = reinterpret_cast<double *>(net->wcrop + 2 * ((nsamples + 1) / 2));   // after the nsamples weights
    cudaMemsetAsync(rsum, 0, nsamples * sizeof(double), s);
    k_crop_rnorm<<<dim3(S - 2 * margin, nsamples), 256, 0, s>>>(S, margin, in, rsum);
    k_crop_rinv<<<(nsamples + 255) / 256, 256, 0, s>>>(nsamples, rsum, net->wcrop);
    cudaMemsetAsync(net->loss, 0, sizeof(double), s);
    k_crop_loss<<<vec_grid(nn), 256, 0, s>>>(nn, (long long)S * S * S, nsamples, net->qf, net->wcrop, net->loss);
    // g = A^T q = L (dinv * q)
    k_crop_flux<<<vec_grid(nc), 256, 0, s>>>(nsamples, S, net->qf, dinv, hcell, net->flux);
    k_crop_node<<<vec_grid(nn), 256, 0, s>>>(nsamples, S, net->flux, nullptr, ox, oy, oz, 0, net->gf);
    k_pack_f32<<<vec_grid(m.nvox()), 256, 0, s>>>(m, net->gf, 1.f, net->g8);
    backward_layers(net, m, s);
    net->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - powf(b1, (float)net->adam_t), bc2 = 1.f - powf(b2, (float)net->adam_t);
    k_adam<<<vec_grid(net->nparams), 256, 0, s>>>(net->nparams, net->params, net->grads, net->adam_m, net->adam_v, lr,
                                                  b1, b2, 1e-8f, bc1, bc2);
    net->launches += 14;
    const int rc = cnn_sync_weights(net, s);
    if (rc != BELLA_OK) return rc;
    if (loss) {
        if (cudaMemcpyAsync(loss, net->loss, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return BELLA_ECUDA;
    }
    return cudaGetLastError() == cudaSuccess ? BELLA_OK : BELLA_ECUDA;
}

int bella_cnn_block(const bella_cnn *net) { return net ? net->block : 0; }

// mode bit 0: linear (no ReLU, no biases); bit 1: bias-free ReLU network.  The
// biases must be zero for either (set_params); they then stay zero in training.
// identity path of the map: output = omega * input + network(input)
int bella_cnn_set_skip(bella_cnn *net, float omega) {
    if (!net || !isfinite(omega)) return BELLA_EINVAL;
    net->omega = omega;
    return BELLA_OK;
}

// the forward, input-gradient and weight-gradient passes on tcgen05 where the staged planes
// fit (1) or on mma.sync and the FP32 CUDA-core loops (0)
int bella_cnn_set_tc(bella_cnn *net, int on) {
    if (!net) return BELLA_EINVAL;
    net->use_tc = on ? 1 : 0;
    return BELLA_OK;
}

// 1 if a tensor-core completion wait gave up since the last call (synchronises), then cleared
int bella_cnn_tc_error(bella_cnn *net) {
    if (!net) return BELLA_EINVAL;
    int h = 0;
    if (cudaMemcpy(&h, net->tc_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return BELLA_ECUDA;
    if (h) cudaMemset(net->tc_err, 0, sizeof(int));
    return h;
}

int bella_cnn_set_mode(bella_cnn *net, int mode) {
    if (!net || mode < 0 || mode > 3) return BELLA_EINVAL;
    net->linear = mode & 1;
    net->bias_free = (mode >> 1) & 1;
    return BELLA_OK;
}

long long bella_cnn_launches(const bella_cnn *net) { return net ? net->launches : 0; }

}  // extern "C"
