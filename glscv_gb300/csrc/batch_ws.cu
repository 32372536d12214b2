// batch_ws.cu -- warp-specialised persistent batched FFT with TMA staging.
//
// Block = 8 compute warps + 1 producer warp.  The producer (one lane) pulls
// (image, pass, tile) items from the plan's work list, waits (bounded) until
// the image's previous pass is complete, and stages the tile into one of
// three shared-memory buffers with the Tensor Memory Accelerator:
//   * a rows tile (LINES contiguous rows) is one cp.async.bulk copy;
//   * a columns tile (W adjacent columns x N rows, W*8 = 32..512 bytes per
//     row) is read as 2-D boxes through a per-image tensor map
//     (cp.async.bulk.tensor.2d) -- the column staging that replaces the
//     reference's separate tiled/untiled copy passes (glsCV/glsCopy.cpp).
// Completion of each copy lands on the stage's "full" mbarrier.  The compute
// warps read their 16 values per thread from the stage, run the Stockham
// passes (exchanging through the same buffer), store to global memory, and
// arrive on the stage's "stored" mbarrier.  The producer then publishes the
// tile (release fence + counter) and refills the stage.  Items are published
// in order, and the producer keeps publishing finished tiles while it waits
// on a dependency, so no block ever holds back the work another waits for.
// Every wait is bounded: on expiry the block records GLSFFT_ERROR_TIMEOUT,
// lets the compute warps drain, waits for its own copies and exits.
#include <cuda.h>

#include "batch_internal.h"
#include "fft_config.h"
#include "fft_kernels.cuh"
#include "glsfft.h"

namespace glsfft {

namespace {

constexpr int kStages = 3;
constexpr int kCompute = 256;                      // compute threads
constexpr int kBlock = kCompute + 32;              // + producer warp
constexpr int kStageElems = 4352;                  // padded_count(4096)
constexpr size_t kStageBytes = kStageElems * sizeof(float2);

struct StageInfo {
    float2 *dst;
    int rows, cols, tile, image;
    int pass, along_rows, flags, scale;
    int valid;  // 0: no more work
    int pad[5];
};

struct WsShared {
    unsigned long long full[kStages];
    unsigned long long stored[kStages];
    StageInfo info[kStages];
};

constexpr size_t kWsSmem = kStages * kStageBytes + sizeof(WsShared) + 128;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long *b, unsigned bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// One try_wait: the thread may be suspended (not spinning on issue slots)
// until the phase completes or a hardware time limit passes.
__device__ __forceinline__ bool mbar_try(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with `parity` to complete; false on expiry.
__device__ bool mbar_wait(unsigned long long *b, unsigned parity, long long limit_ns) {
    if (mbar_try(b, parity)) return true;
    const unsigned long long t0 = gtimer();
    for (unsigned it = 0; it < (1u << 24); it++) {
        if (mbar_try(b, parity)) return true;
        if ((long long)(gtimer() - t0) > limit_ns) return false;
    }
    return false;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tensor2d_g2s(void *dst, const void *tmap, int x, int y,
                                             unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// ------------------------------------------------------------ compute side
template <int N>
__device__ __forceinline__ void ws_rows(float2 *stage, const StageInfo &in, const float2 *tw,
                                        int tid) {
    constexpr int E = 16, T = N / E, LINES = kCompute / T;
    const int l = tid / T, t = tid % T;
    const int row = in.tile * LINES + l;
    const bool active = row < in.rows;
    const bool cin = in.flags & PF_CONJ_IN, cout = in.flags & PF_CONJ_OUT;
    float2 x[E];
    const float2 *sp = stage + l * N + t;
#pragma unroll
    for (int m = 0; m < E; m++) x[m] = active ? sp[m * T] : make_float2(0.f, 0.f);
    conj_line(x, cin);
    SyncCompute256{}();  // the exchanges below overwrite the staged tile
    LineFft<N, E, SyncCompute256>::run(x, t, RowSm{stage + l * padded_count(N)}, tw);
    finish_line(x, in.scale ? 1.0f / (float)N : 1.0f, cout);
    if (active) store_line<N, E, T>(in.dst + (size_t)row * N, 1, x, t, in.flags & PF_SHIFT_COLS);
}

template <int N>
__device__ __forceinline__ void ws_cols(float2 *stage, const StageInfo &in, const float2 *tw,
                                        int tid) {
    constexpr int E = 16, T = N / E, W = kCompute / T;
    const int c = tid % W, t = tid / W;
    const int col = in.tile * W + c;
    const bool active = col < in.cols;
    const bool cin = in.flags & PF_CONJ_IN, cout = in.flags & PF_CONJ_OUT;
    float2 x[E];
    const float2 *sp = stage + t * W + c;  // out-of-range columns were zero-filled
#pragma unroll
    for (int m = 0; m < E; m++) x[m] = sp[m * T * W];
    conj_line(x, cin);
    SyncCompute256{}();
    LineFft<N, E, SyncCompute256>::run(x, t, ColSm<W>{stage, c}, tw);
    finish_line(x, in.scale ? 1.0f / (float)N : 1.0f, cout);
    if (active) store_line<N, E, T>(in.dst + col, (size_t)in.cols, x, t, in.flags & PF_SHIFT_ROWS);
}

__device__ __forceinline__ void ws_compute(float2 *stage, const StageInfo &in, const float2 *tw, int tid) {
    if (in.along_rows) {
        switch (in.cols) {
        case 16: ws_rows<16>(stage, in, tw, tid); break;
        case 32: ws_rows<32>(stage, in, tw, tid); break;
        case 64: ws_rows<64>(stage, in, tw, tid); break;
        case 128: ws_rows<128>(stage, in, tw, tid); break;
        case 256: ws_rows<256>(stage, in, tw, tid); break;
        case 512: ws_rows<512>(stage, in, tw, tid); break;
        case 1024: ws_rows<1024>(stage, in, tw, tid); break;
        case 2048: ws_rows<2048>(stage, in, tw, tid); break;
        case 4096: ws_rows<4096>(stage, in, tw, tid); break;
        default: break;
        }
    } else {
        switch (in.rows) {
        case 16: ws_cols<16>(stage, in, tw, tid); break;
        case 32: ws_cols<32>(stage, in, tw, tid); break;
        case 64: ws_cols<64>(stage, in, tw, tid); break;
        case 128: ws_cols<128>(stage, in, tw, tid); break;
        case 256: ws_cols<256>(stage, in, tw, tid); break;
        case 512: ws_cols<512>(stage, in, tw, tid); break;
        case 1024: ws_cols<1024>(stage, in, tw, tid); break;
        default: break;
        }
    }
}

}  // namespace

template <int MINB>
__global__ void __launch_bounds__(kBlock, MINB) fft_batch_ws(BatchArgs a) {
    extern __shared__ __align__(128) unsigned char ws_raw[];
    // 128-byte aligned stage buffers, then the barriers and stage records
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(ws_raw) + 127) & ~uintptr_t(127));
    float2 *stages = reinterpret_cast<float2 *>(base);
    WsShared &sh = *reinterpret_cast<WsShared *>(base + kStages * kStageBytes);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(&sh.full[s], 1);
            mbar_init(&sh.stored[s], kCompute);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (threadIdx.x >= kCompute) {
        // ------------------------------------------------------ producer
        if (threadIdx.x != kCompute) return;
        const int tile_px = kBatchTileElems;
        constexpr int kChunk = 4;  // items claimed per queue atomic
        int issued = 0, published = 0;
        bool failed = false;
        // Publish the stored items [published, end) in order: one release
        // fence, then one counter add per run of the same (image, pass).  A
        // stage's record still describes its item until the item is
        // published (the stage is refilled only after that).
        auto publish_upto = [&](int end) {
            if (end <= published) return;
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            while (published < end) {
                const int img = sh.info[published % kStages].image;
                const int pas = sh.info[published % kStages].pass;
                unsigned n = 0;
                while (published < end && sh.info[published % kStages].image == img &&
                       sh.info[published % kStages].pass == pas) {
                    published++;
                    n++;
                }
                atomicAdd(a.done + img * kBatchMaxPasses + pas, n);
            }
        };
        // publish every issued item whose tile the compute warps have stored
        auto service = [&]() {
            int end = published;
            while (end < issued && mbar_test(&sh.stored[end % kStages], (end / kStages) & 1)) end++;
            publish_upto(end);
        };
        const int chunk = a.claim_chunk < 1 ? 1 : (a.claim_chunk > kChunk ? kChunk : a.claim_chunk);
        unsigned claim = atomicAdd(a.head, (unsigned)chunk);
        int cur_img = -1, cur_pass = -1, cur_need = -1;
        bool dep_ok = false;
        BatchImage im{};
        BatchPass ps{};
        for (;;) {
            const int base = (int)claim;
            const bool done = base >= a.n_items || *(volatile int *)a.error;
            if (!done && a.claim_ahead) claim = atomicAdd(a.head, (unsigned)chunk);  // in flight
            const int cnt = done ? 0 : min(chunk, a.n_items - base);
            BatchItem its[kChunk];
#pragma unroll
            for (int q = 0; q < kChunk; q++)
                if (q < cnt) its[q] = a.items[base + q];
#pragma unroll
            for (int q = 0; q <= kChunk; q++) {
                if (q > cnt || (q == cnt && !done)) break;
                const int s = issued % kStages;
                // the stage's previous item must be stored (and is then published)
                while (published <= issued - kStages) {
                    if (!mbar_wait(&sh.stored[published % kStages], (published / kStages) & 1,
                                   a.wait_limit_ns)) {
                        failed = true;
                        break;
                    }
                    service();
                }
                if (failed) break;
                StageInfo &inf = sh.info[s];
                if (q == cnt) {  // queue exhausted: tell the compute warps to stop
                    inf.valid = 0;
                    mbar_arrive(&sh.full[s]);
                    break;
                }
                const BatchItem it = its[q];
                if (it.image != cur_img || it.pass != cur_pass || it.need != cur_need) {
                    if (it.image != cur_img) im = a.images[it.image];
                    if (it.pass != cur_pass) ps = a.passes[it.pass];
                    cur_img = it.image;
                    cur_pass = it.pass;
                    cur_need = it.need;
                    dep_ok = it.pass == 0;
                }
                if (!dep_ok) {
                    // every tile of this image's previous pass must be published
                    const unsigned *cnt_p = a.done + it.image * kBatchMaxPasses + it.pass - 1;
                    const unsigned long long t0 = gtimer();
                    while (ld_acquire_u32(cnt_p) < (unsigned)it.need) {
                        service();
                        if ((long long)(gtimer() - t0) > a.wait_limit_ns) {
                            failed = true;
                            break;
                        }
                        __nanosleep(128);
                    }
                    if (failed) break;
                    // order the acquire before the async-proxy (TMA) reads
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                    dep_ok = true;
                }
                inf.dst = im.dst;
                inf.rows = im.rows;
                inf.cols = im.cols;
                inf.tile = it.tile;
                inf.image = it.image;
                inf.pass = it.pass;
                inf.along_rows = ps.along_rows;
                inf.flags = ps.flags;
                inf.scale = ps.scale;
                inf.valid = 1;
                float2 *stage = stages + (size_t)s * kStageElems;
                if (ps.along_rows) {
                    const int n = im.cols, lines = tile_px / n;
                    const int row0 = it.tile * lines;
                    const int nrows = min(lines, im.rows - row0);
                    const unsigned bytes = (unsigned)(nrows * n * sizeof(float2));
                    const float2 *src = (it.pass == 0 ? im.src : im.dst) + (size_t)row0 * n;
                    mbar_arrive_tx(&sh.full[s], bytes);
                    bulk_g2s(stage, src, bytes, &sh.full[s]);
                } else {
                    const int n = im.rows, w = tile_px / n;
                    const int br = n < 256 ? n : 256;
                    const void *tmap =
                        static_cast<const unsigned char *>(a.tmaps) + (size_t)it.image * 128;
                    mbar_arrive_tx(&sh.full[s], (unsigned)(n * w * sizeof(float2)));
                    for (int b = 0; b < n / br; b++)
                        tensor2d_g2s(stage + (size_t)b * br * w, tmap, it.tile * w, b * br,
                                     &sh.full[s]);
                }
                issued++;
                service();
            }
            if (failed || done) break;
            if (!a.claim_ahead) claim = atomicAdd(a.head, (unsigned)chunk);
        }
        if (failed) {
            atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
            // the compute warps finish what was issued, then stop here
            const int s = issued % kStages;
            sh.info[s].valid = 0;
            mbar_arrive(&sh.full[s]);
        }
        // publish what is left, and make sure no copy into this block's
        // shared memory is still in flight when the block exits
        while (published < issued) {
            const int j = published;
            if (mbar_wait(&sh.stored[j % kStages], (j / kStages) & 1, a.wait_limit_ns)) {
                publish_upto(j + 1);
            } else {
                atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
                mbar_wait(&sh.full[j % kStages], (j / kStages) & 1, a.wait_limit_ns);
                published++;
            }
        }
        return;
    }

    // ------------------------------------------------------------ compute
    const int tid = threadIdx.x;
    for (int k = 0;; k++) {
        const int s = k % kStages;
        if (!mbar_wait(&sh.full[s], (k / kStages) & 1, a.wait_limit_ns)) {
            if (tid == 0) atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
            break;
        }
        const StageInfo in = sh.info[s];
        if (!in.valid) break;
        ws_compute(stages + (size_t)s * kStageElems, in, a.tw, tid);
        // generic-proxy writes to the stage happen before the next TMA write
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&sh.stored[s]);
    }
}

template <int MINB>
static cudaError_t prepare_ws() {
    static cudaError_t once = cudaFuncSetAttribute(
        fft_batch_ws<MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWsSmem);
    return once;
}

cudaError_t launch_batch_ws(const BatchArgs &a, int grid, int blocks_per_sm, cudaStream_t s) {
    cudaError_t e = blocks_per_sm >= 2 ? prepare_ws<2>() : prepare_ws<1>();
    if (e != cudaSuccess) return e;
    if (blocks_per_sm >= 2) fft_batch_ws<2><<<grid, kBlock, kWsSmem, s>>>(a);
    else fft_batch_ws<1><<<grid, kBlock, kWsSmem, s>>>(a);
    return cudaGetLastError();
}

int batch_ws_grid(int device, int blocks_per_sm) {
    cudaError_t e = blocks_per_sm >= 2 ? prepare_ws<2>() : prepare_ws<1>();
    if (e != cudaSuccess) return 0;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return 0;
    e = blocks_per_sm >= 2
            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fft_batch_ws<2>, kBlock, kWsSmem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fft_batch_ws<1>, kBlock, kWsSmem);
    if (e != cudaSuccess) return 0;
    if (per_sm > blocks_per_sm) per_sm = blocks_per_sm;
    return sms * (per_sm > 0 ? per_sm : 1);
}

}  // namespace glsfft
