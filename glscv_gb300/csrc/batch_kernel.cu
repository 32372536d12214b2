// batch_kernel.cu -- persistent batched 2-D FFT over images of mixed sizes.
//
// One launch processes a whole plan.  Resident blocks pull (image, pass,
// tile) work items from a global counter; a pass of an image may start only
// when every tile of that image's previous pass is complete (a per-image
// counter; the wait is bounded by a globaltimer deadline, after which the
// block records GLSFFT_ERROR_TIMEOUT and moves on).  The host orders the
// item list so that an image's next pass is dispensed about one resident
// grid of items after its previous pass: the data it reads has just been
// written and is still in the 129 MB L2, so a chained 2-D FFT touches HBM
// about once per read and once per write of the image instead of once per
// pass.  Replaces the reference's one-draw-per-pass-per-tile loop
// (glsCV/glsFft.cpp:561-652) for many images at once.
#include "batch_internal.h"
#include "fft_config.h"
#include "fft_kernels.cuh"
#include "glsfft.h"

namespace glsfft {

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Spin until *p >= need; false when the deadline passes first.  A second,
// iteration-count bound backs up the timer.
__device__ bool bounded_wait(const unsigned *p, unsigned need, long long limit_ns) {
    if (ld_acquire(p) >= need) return true;
    const unsigned long long t0 = global_ns();
    unsigned sleep = 32;
    for (unsigned it = 0; it < (1u << 26); it++) {
        __nanosleep(sleep);
        if (sleep < 2048) sleep <<= 1;
        if (ld_acquire(p) >= need) return true;
        if ((long long)(global_ns() - t0) > limit_ns) return false;
    }
    return false;
}

template <bool FIRST>
__device__ __forceinline__ float2 load_c2(const float2 *p) {
    // pass 0 reads the plan's input (never written by this launch before it
    // is read); later passes read data other blocks wrote during this launch,
    // so they bypass L1 (ld.global.cg)
    if constexpr (FIRST) return __ldg(p);
    else return __ldcg(p);
}

template <int N, bool FIRST>
__device__ __forceinline__ void batch_rows_tile(const BatchImage &im, const BatchPass &ps,
                                                int tile, const float2 *tw, float2 *smem) {
    constexpr int E = 16, T = N / E, LINES = kBatchThreads / T;
    const int l = threadIdx.x / T, t = threadIdx.x % T;
    const int row = tile * LINES + l;
    const bool active = row < im.rows;
    const float2 *src = FIRST ? im.src : im.dst;
    const bool cin = ps.flags & PF_CONJ_IN, cout = ps.flags & PF_CONJ_OUT;
    float2 x[E];
#pragma unroll
    for (int m = 0; m < E; m++)
        x[m] = active ? load_c2<FIRST>(src + (size_t)row * N + t + m * T) : make_float2(0.f, 0.f);
    conj_line(x, cin);
    LineFft<N, E>::run(x, t, RowSm{smem + l * padded_count(N)}, tw);
    finish_line(x, ps.scale ? 1.0f / (float)N : 1.0f, cout);
    if (active) store_line<N, E, T>(im.dst + (size_t)row * N, 1, x, t, ps.flags & PF_SHIFT_COLS);
}

template <int N, bool FIRST>
__device__ __forceinline__ void batch_cols_tile(const BatchImage &im, const BatchPass &ps,
                                                int tile, const float2 *tw, float2 *smem) {
    constexpr int E = 16, T = N / E, W = kBatchThreads / T;
    const int c = threadIdx.x % W, t = threadIdx.x / W;
    const int cols = im.cols;
    const int col = tile * W + c;
    const bool active = col < cols;
    const float2 *src = FIRST ? im.src : im.dst;
    const bool cin = ps.flags & PF_CONJ_IN, cout = ps.flags & PF_CONJ_OUT;
    float2 x[E];
#pragma unroll
    for (int m = 0; m < E; m++)
        x[m] = active ? load_c2<FIRST>(src + (size_t)(t + m * T) * cols + col) : make_float2(0.f, 0.f);
    conj_line(x, cin);
    LineFft<N, E>::run(x, t, ColSm<W>{smem, c}, tw);
    finish_line(x, ps.scale ? 1.0f / (float)N : 1.0f, cout);
    if (active) store_line<N, E, T>(im.dst + col, (size_t)cols, x, t, ps.flags & PF_SHIFT_ROWS);
}

template <bool FIRST>
__device__ void batch_item(const BatchImage &im, const BatchPass &ps, int tile,
                           const float2 *tw, float2 *smem) {
    if (ps.along_rows) {
        switch (im.cols) {
        case 16: batch_rows_tile<16, FIRST>(im, ps, tile, tw, smem); break;
        case 32: batch_rows_tile<32, FIRST>(im, ps, tile, tw, smem); break;
        case 64: batch_rows_tile<64, FIRST>(im, ps, tile, tw, smem); break;
        case 128: batch_rows_tile<128, FIRST>(im, ps, tile, tw, smem); break;
        case 256: batch_rows_tile<256, FIRST>(im, ps, tile, tw, smem); break;
        case 512: batch_rows_tile<512, FIRST>(im, ps, tile, tw, smem); break;
        case 1024: batch_rows_tile<1024, FIRST>(im, ps, tile, tw, smem); break;
        case 2048: batch_rows_tile<2048, FIRST>(im, ps, tile, tw, smem); break;
        case 4096: batch_rows_tile<4096, FIRST>(im, ps, tile, tw, smem); break;
        default: break;
        }
    } else {
        switch (im.rows) {
        case 16: batch_cols_tile<16, FIRST>(im, ps, tile, tw, smem); break;
        case 32: batch_cols_tile<32, FIRST>(im, ps, tile, tw, smem); break;
        case 64: batch_cols_tile<64, FIRST>(im, ps, tile, tw, smem); break;
        case 128: batch_cols_tile<128, FIRST>(im, ps, tile, tw, smem); break;
        case 256: batch_cols_tile<256, FIRST>(im, ps, tile, tw, smem); break;
        case 512: batch_cols_tile<512, FIRST>(im, ps, tile, tw, smem); break;
        case 1024: batch_cols_tile<1024, FIRST>(im, ps, tile, tw, smem); break;
        default: break;
        }
    }
}

__global__ void __launch_bounds__(kBatchThreads, 2) fft_batch_persistent(BatchArgs a) {
    extern __shared__ float4 smem_raw[];
    float2 *smem = reinterpret_cast<float2 *>(smem_raw);
    __shared__ int s_idx;
    __shared__ int s_skip;
    for (;;) {
        if (threadIdx.x == 0) {
            s_idx = (int)atomicAdd(a.head, 1u);
            s_skip = 0;
        }
        __syncthreads();
        const int idx = s_idx;
        if (idx >= a.n_items) break;
        const BatchItem it = a.items[idx];
        if (threadIdx.x == 0) {
            if (*(volatile int *)a.error) {
                s_skip = 1;  // an earlier wait expired: drain the queue quickly
            } else if (it.pass > 0 &&
                       !bounded_wait(a.done + it.image * kBatchMaxPasses + it.pass - 1,
                                     (unsigned)it.need, a.wait_limit_ns)) {
                atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
                s_skip = 1;
            }
        }
        __syncthreads();
        if (!s_skip) {
            const BatchImage im = a.images[it.image];
            const BatchPass ps = a.passes[it.pass];
            if (it.pass == 0) batch_item<true>(im, ps, it.tile, a.tw, smem);
            else batch_item<false>(im, ps, it.tile, a.tw, smem);
        }
        __syncthreads();  // every thread's stores of this tile are issued
        if (threadIdx.x == 0) {
            __threadfence();  // release them before the count (grid-sync pattern)
            atomicAdd(a.done + it.image * kBatchMaxPasses + it.pass, 1u);
        }
    }
}

constexpr size_t kBatchSmem = sizeof(float2) * (size_t)padded_count(kBatchTileElems);

cudaError_t launch_batch_persistent(const BatchArgs &a, int grid, cudaStream_t s) {
    fft_batch_persistent<<<grid, kBatchThreads, kBatchSmem, s>>>(a);
    return cudaGetLastError();
}

int batch_persistent_grid(int device) {
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fft_batch_persistent,
                                                      kBatchThreads, kBatchSmem) != cudaSuccess)
        return 0;
    return sms * (per_sm > 0 ? per_sm : 1);
}

bool batch_supported(int rows, int cols) {
    return rows >= 16 && rows <= 1024 && cols >= 16 && cols <= 4096;
}

}  // namespace glsfft
