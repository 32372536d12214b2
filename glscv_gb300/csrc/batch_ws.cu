// batch_ws.cu -- warp-specialised persistent batched FFT with TMA staging.
//
// Block = 8 compute warps + a loader warp + a storer warp (one active lane
// each).  The loader pulls (image, pass, tile) items from the plan's work
// list, waits (bounded) until the image's previous pass is complete, and
// stages the tile into a shared-memory ring with the Tensor Memory
// Accelerator:
//   * a rows tile (LINES contiguous rows) is one cp.async.bulk copy;
//   * a columns tile (W adjacent columns x N rows, W*8 = 32..512 bytes per
//     row) is one cp.async.bulk copy of a contiguous block when the image
//     has a column-tiled workspace (BatchImage::work; the rows pass before
//     stored its tile there with one 3-D tensor box), else 2-D boxes through
//     a per-image tensor map of dst (cp.async.bulk.tensor.2d) -- the column
//     staging that replaces the reference's separate tiled/untiled copy
//     passes (glsCV/glsCopy.cpp);
//   * an image whose intermediates all stay in the workspace
//     (BatchImage::ws_inplace) loads a later rows tile as one 128-byte-
//     swizzled 2-D box of 256 pieces and stores its columns blocks back in
//     place with cp.async.bulk.
// Completion of each copy lands on the stage's "full" mbarrier.  The compute
// warps read their 16 values per thread from the stage, run the Stockham
// passes (exchanging through the same buffer), write the results back into
// the stage in the image's layout and arrive on the stage's "computed"
// mbarrier.  The storer writes the tile out with the TMA (one cp.async.bulk
// for a rows tile, or one 3-D tensor box into the workspace; 2-D tensor
// boxes for a columns tile), arrives on the
// stage's "empty" mbarrier as soon as the store has read the stage (the
// loader then refills it), waits for the store's writes and publishes the
// tile at once (release fence + counter), so dependent passes never wait on
// a block's later work.  Every wait is bounded: on expiry the block records
// GLSFFT_ERROR_TIMEOUT, lets the compute warps drain, waits for its own
// copies and exits.
#include <cuda.h>

#include "batch_internal.h"
#include "fft_config.h"
#include "fft_kernels.cuh"
#include "glsfft.h"
#include "tma_device.cuh"

namespace glsfft {

namespace {

constexpr int kCompute = 256;                      // compute threads
constexpr int kLoaderWarp = kCompute / 32;         // warp 8
constexpr int kStorerWarp = kCompute / 32 + 1;     // warp 9
constexpr int kBlock = kCompute + 64;              // + loader and storer warps
constexpr int kStageElems = 4352;                  // padded_count(4096)
constexpr size_t kStageBytes = kStageElems * sizeof(float2);

struct StageInfo {
    float2 *dst;
    float2 *work;  // the image's column-tiled workspace, or null
    int rows, cols, tile, image;
    int pass, along_rows, flags, scale;
    int valid;       // 0: no more work
    int ws_inplace;  // the image keeps its intermediates in work (BatchImage)
    int last;        // the image's last pass
    int pad;
};

template <int ST>
struct WsShared {
    unsigned long long full[ST];      // tile staged (TMA transaction bytes)
    unsigned long long computed[ST];  // results in the stage (256 compute arrivals)
    unsigned long long empty[ST];     // the store has read the stage (storer)
    StageInfo info[ST];
    unsigned long long st[6];  // timing sums when BatchArgs::stats is set (BS_* order)
};

// Shared-memory copy of the twiddle tables of the current line length, for
// lengths 32..1024 (longer lines read the global tables).
constexpr int kTwCacheMax = 1024;
constexpr int kTwCacheF4 = tw_smem_float4(kTwCacheMax);
__host__ __device__ constexpr bool tw_cached(int n) { return n >= 32 && n <= kTwCacheMax; }

// dynamic shared memory of a block with ST stages
template <int ST>
constexpr size_t ws_smem() {
    return ST * kStageBytes + kTwCacheF4 * sizeof(float4) + sizeof(WsShared<ST>) + 1024;
}

// ------------------------------------------------------------ compute side
// the line engine with the shared-memory tables where the length has them
template <int N, class Sm>
__device__ __forceinline__ void ws_line(float2 (&x)[16 < N ? 16 : N], int t, Sm sm,
                                        const float2 *tw, const float4 *twc) {
    constexpr int E = 16 < N ? 16 : N;
    if constexpr (tw_cached(N)) {
        static_assert(tw_smem_ok(N) && tw_smem_float4(N) <= kTwCacheF4, "twiddle cache layout");
        LineFft<N, E, SyncCompute256>::run(x, t, sm, SmemTw<N>{twc});
    } else {
        LineFft<N, E, SyncCompute256>::run(x, t, sm, tw);
    }
}

template <int N>
__device__ __forceinline__ void ws_rows(float2 *stage, const StageInfo &in, const float2 *tw,
                                        const float4 *twc, int tid) {
    constexpr int E = 16, T = N / E, LINES = kCompute / T;
    const int l = tid / T, t = tid % T;
    const int row = in.tile * LINES + l;
    const bool active = row < in.rows;
    const bool cin = in.flags & PF_CONJ_IN, cout = in.flags & PF_CONJ_OUT;
    // an in-place workspace image: passes after the first stage the tile
    // in the workspace box's order
    float2 x[E];
    if (N >= 1024 && in.ws_inplace && in.pass > 0) {
        const unsigned p0 = ws_swz_base(N, l, t);
#pragma unroll
        for (int m = 0; m < E; m++) x[m] = stage[p0 + 256 * m];
    } else {
        const float2 *sp = stage + l * N + t;
#pragma unroll
        for (int m = 0; m < E; m++) x[m] = active ? sp[m * T] : make_float2(0.f, 0.f);
    }
    conj_line(x, cin);
    SyncCompute256{}();  // the exchanges below overwrite the staged tile
    ws_line<N>(x, t, RowSm{stage + l * padded_count(N)}, tw, twc);
    finish_line(x, in.scale ? 1.0f / (float)N : 1.0f, cout);
    // results back into the stage as the tile's rows, contiguous, for the
    // producer's bulk store or 3-D box (after every thread's last exchange
    // read)
    SyncCompute256{}();
    if (active) store_line<N, E, T>(stage + l * N, 1, x, t, in.flags & PF_SHIFT_COLS);
}

template <int N>
__device__ __forceinline__ void ws_cols(float2 *stage, const StageInfo &in, const float2 *tw,
                                        const float4 *twc, int tid) {
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
    ws_line<N>(x, t, ColSm<W>{stage, c}, tw, twc);
    finish_line(x, in.scale ? 1.0f / (float)N : 1.0f, cout);
    // results back into the stage as the tensor-map box ([position][W]);
    // columns past the image edge are clipped by the tensor store
    (void)active;
    SyncCompute256{}();
    store_line<N, E, T>(stage + c, (size_t)W, x, t, in.flags & PF_SHIFT_ROWS);
}

// Reload the shared-memory tables when the line length changes (every
// compute thread sees the same items, so `cached_n` agrees across threads).
__device__ __forceinline__ void tw_cache_for(int n, const float2 *tw, float4 *twc, int tid,
                                             int &cached_n) {
    if (n == cached_n || !tw_cached(n)) return;
    SyncCompute256{}();  // every compute thread is done with the previous tables
    switch (n) {
    case 32: tw_fill_smem<32>(twc, tw, tid, kCompute); break;
    case 64: tw_fill_smem<64>(twc, tw, tid, kCompute); break;
    case 128: tw_fill_smem<128>(twc, tw, tid, kCompute); break;
    case 256: tw_fill_smem<256>(twc, tw, tid, kCompute); break;
    case 512: tw_fill_smem<512>(twc, tw, tid, kCompute); break;
    case 1024: tw_fill_smem<1024>(twc, tw, tid, kCompute); break;
    default: break;
    }
    SyncCompute256{}();
    cached_n = n;
}

__device__ __forceinline__ void ws_compute(float2 *stage, const StageInfo &in, const float2 *tw,
                                           float4 *twc, int tid, int &cached_n) {
    tw_cache_for(in.along_rows ? in.cols : in.rows, tw, twc, tid, cached_n);
    if (in.along_rows) {
        switch (in.cols) {
        case 16: ws_rows<16>(stage, in, tw, twc, tid); break;
        case 32: ws_rows<32>(stage, in, tw, twc, tid); break;
        case 64: ws_rows<64>(stage, in, tw, twc, tid); break;
        case 128: ws_rows<128>(stage, in, tw, twc, tid); break;
        case 256: ws_rows<256>(stage, in, tw, twc, tid); break;
        case 512: ws_rows<512>(stage, in, tw, twc, tid); break;
        case 1024: ws_rows<1024>(stage, in, tw, twc, tid); break;
        case 2048: ws_rows<2048>(stage, in, tw, twc, tid); break;
        case 4096: ws_rows<4096>(stage, in, tw, twc, tid); break;
        default: break;
        }
    } else {
        switch (in.rows) {
        case 16: ws_cols<16>(stage, in, tw, twc, tid); break;
        case 32: ws_cols<32>(stage, in, tw, twc, tid); break;
        case 64: ws_cols<64>(stage, in, tw, twc, tid); break;
        case 128: ws_cols<128>(stage, in, tw, twc, tid); break;
        case 256: ws_cols<256>(stage, in, tw, twc, tid); break;
        case 512: ws_cols<512>(stage, in, tw, twc, tid); break;
        case 1024: ws_cols<1024>(stage, in, tw, twc, tid); break;
        default: break;
        }
    }
}

}  // namespace

template <int MINB, int ST>
__global__ void __launch_bounds__(kBlock, MINB) fft_batch_ws(BatchArgs a) {
    extern __shared__ __align__(128) unsigned char ws_raw[];
    // 1024-byte aligned stage buffers (the 128-byte swizzle of the
    // in-place workspace boxes follows shared-memory address bits 7-9), the
    // twiddle cache, then the barriers and stage records (offsetting the
    // shared array itself, not a cast integer, keeps the compiler's
    // shared-window addressing)
    unsigned char *base = ws_raw + ((1024u - (smem_u32(ws_raw) & 1023u)) & 1023u);
    float2 *stages = reinterpret_cast<float2 *>(base);
    float4 *twc = reinterpret_cast<float4 *>(base + ST * kStageBytes);
    WsShared<ST> &sh = *reinterpret_cast<WsShared<ST> *>(base + ST * kStageBytes +
                                                         kTwCacheF4 * sizeof(float4));

    if (threadIdx.x == 0) {
        for (int i = 0; i < 6; i++) sh.st[i] = 0;
        for (int s = 0; s < ST; s++) {
            mbar_init(&sh.full[s], 1);
            mbar_init(&sh.computed[s], kCompute);
            mbar_init(&sh.empty[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int warp = threadIdx.x / 32;

    if (warp == kLoaderWarp) {
        // -------------------------------------------------------- loader
        if (threadIdx.x % 32 != 0) return;
        const int tile_px = kBatchTileElems;
        constexpr int kChunk = 4;  // items claimed per queue atomic
        if (a.stats) sh.st[BS_PRODUCER_TOTAL] = gtimer();
        int issued = 0;
        bool failed = false;
        int cur_img = -1, cur_pass = -1, cur_need = -1;
        bool dep_ok = false;
        BatchImage im{};
        BatchPass ps{};
        // Issue one item into the next stage, or the stop record (itp null).
        // `pre` is the item's image record when the caller fetched it ahead;
        // `spec` a relaxed look at its dependency counter (UINT_MAX: none).
        // The item's records and dependency come first, so their latency
        // overlaps the compute warps' work on the stages in flight; then
        // the stage is waited for.  Returns false when a wait expired.
        auto issue_item = [&](const BatchItem *itp, const BatchImage *pre, unsigned spec) -> bool {
            const int s = issued % ST;
            if (itp) {
                const BatchItem &it = *itp;
                if (it.image != cur_img || it.pass != cur_pass || it.need != cur_need) {
                    if (it.image != cur_img) im = pre ? *pre : a.images[it.image];
                    if (it.pass != cur_pass) ps = a.passes[it.pass];
                    cur_img = it.image;
                    cur_pass = it.pass;
                    cur_need = it.need;
                    dep_ok = it.pass == 0;
                }
                if (!dep_ok && spec != 0xffffffffu && spec >= (unsigned)it.need) {
                    // the relaxed read saw every tile published: make it an acquire
                    asm volatile("fence.acq_rel.gpu;" ::: "memory");
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                    dep_ok = true;
                }
                if (!dep_ok) {
                    // every tile of this image's previous pass must be published
                    const unsigned *cnt_p = a.done + it.image * kBatchMaxPasses + it.pass - 1;
                    const unsigned long long t0 = gtimer();
                    bool ok = true;
                    while (ld_acquire_u32(cnt_p) < (unsigned)it.need) {
                        if ((long long)(gtimer() - t0) > a.wait_limit_ns) {
                            ok = false;
                            break;
                        }
                        __nanosleep(64);
                    }
                    if (a.stats) sh.st[BS_DEP_WAIT] += gtimer() - t0;
                    if (!ok) return false;
                    // order the acquire before the async-proxy (TMA) reads
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                    dep_ok = true;
                }
            }
            // the store of the stage's previous item must have read it
            if (issued >= ST) {
                const unsigned long long tr0 = a.stats ? gtimer() : 0;
                const int j = issued - ST;
                if (!mbar_wait(&sh.empty[s], (j / ST) & 1, a.wait_limit_ns)) return false;
                if (a.stats) sh.st[BS_REFILL_WAIT] += gtimer() - tr0;
            }
            StageInfo &inf = sh.info[s];
            if (!itp) {  // queue exhausted: tell the compute warps and the storer to stop
                inf.valid = 0;
                mbar_arrive(&sh.full[s]);
                issued++;
                return true;
            }
            const BatchItem &it = *itp;
            inf.dst = im.dst;
            inf.work = im.work;
            inf.rows = im.rows;
            inf.cols = im.cols;
            inf.tile = it.tile;
            inf.image = it.image;
            inf.pass = it.pass;
            inf.along_rows = ps.along_rows;
            inf.flags = ps.flags;
            inf.scale = ps.scale;
            inf.valid = 1;
            inf.ws_inplace = im.ws_inplace;
            inf.last = it.pass == a.n_passes - 1;
            float2 *stage = stages + (size_t)s * kStageElems;
            if (ps.along_rows && im.ws_inplace && it.pass > 0) {
                // the tile's 256 pieces of 128 bytes from the workspace
                const void *tmap = static_cast<const unsigned char *>(a.tmaps) +
                                   (size_t)it.image * 128 * kBatchTmapsPerImage + 256;
                mbar_arrive_tx(&sh.full[s], (unsigned)(tile_px * sizeof(float2)));
                tensor2d_g2s(stage, tmap, it.tile * 16, 0, &sh.full[s]);
            } else if (ps.along_rows) {
                const int n = im.cols, lines = tile_px / n;
                const int row0 = it.tile * lines;
                const int nrows = min(lines, im.rows - row0);
                const unsigned bytes = (unsigned)(nrows * n * sizeof(float2));
                const float2 *src = (it.pass == 0 ? im.src : im.dst) + (size_t)row0 * n;
                mbar_arrive_tx(&sh.full[s], bytes);
                bulk_g2s(stage, src, bytes, &sh.full[s]);
            } else if (im.work) {
                // the previous rows pass left this tile as one contiguous block
                const int n = im.rows, w = tile_px / n;
                const unsigned bytes = (unsigned)(n * w * sizeof(float2));
                mbar_arrive_tx(&sh.full[s], bytes);
                bulk_g2s(stage, im.work + (size_t)it.tile * n * w, bytes, &sh.full[s]);
            } else {
                const int n = im.rows, w = tile_px / n;
                const int br = n < 256 ? n : 256;
                const void *tmap = static_cast<const unsigned char *>(a.tmaps) +
                                   (size_t)it.image * 128 * kBatchTmapsPerImage;
                mbar_arrive_tx(&sh.full[s], (unsigned)(n * w * sizeof(float2)));
                for (int b = 0; b < n / br; b++)
                    tensor2d_g2s(stage + (size_t)b * br * w, tmap, it.tile * w, b * br, &sh.full[s]);
            }
            issued++;
            return true;
        };

        if (a.claim_ahead >= 2) {
            // Deep prefetch, one item per claim: item k+3 is claimed, item
            // k+2's record fetched, and item k+1's image record and
            // dependency counter read, while item k is issued -- each load
            // has a whole item's time to arrive.
            const unsigned n = (unsigned)a.n_items;
            const unsigned none = 0xffffffffu;
            unsigned c0 = atomicAdd(a.head, 1u), c1 = atomicAdd(a.head, 1u);
            unsigned c2 = atomicAdd(a.head, 1u);
            BatchItem r0{}, r1{};
            if (c0 < n) r0 = a.items[c0];
            if (c1 < n) r1 = a.items[c1];
            BatchImage i0{};
            unsigned s0 = none;
            if (c0 < n) {
                i0 = a.images[r0.image];
                if (r0.pass > 0) s0 = ld_relaxed_u32(a.done + r0.image * kBatchMaxPasses + r0.pass - 1);
            }
            int err = 0;
            for (;;) {
                if (c0 >= n || err) {
                    if (!issue_item(nullptr, nullptr, none)) failed = true;
                    break;
                }
                const unsigned c3 = c2 < n ? atomicAdd(a.head, 1u) : n;
                BatchItem r2{};
                if (c2 < n) r2 = a.items[c2];
                BatchImage i1{};
                unsigned s1 = none;
                if (c1 < n) {
                    i1 = a.images[r1.image];
                    if (r1.pass > 0)
                        s1 = ld_relaxed_u32(a.done + r1.image * kBatchMaxPasses + r1.pass - 1);
                }
                const int err1 = ld_relaxed_s32(a.error);
                if (!issue_item(&r0, &i0, s0)) {
                    failed = true;
                    break;
                }
                c0 = c1;
                c1 = c2;
                c2 = c3;
                r0 = r1;
                r1 = r2;
                i0 = i1;
                s0 = s1;
                err = err1;
            }
        } else {
            const int chunk =
                a.claim_chunk < 1 ? 1 : (a.claim_chunk > kChunk ? kChunk : a.claim_chunk);
            unsigned claim = atomicAdd(a.head, (unsigned)chunk);
            for (;;) {
                const int base_i = (int)claim;
                const bool done = base_i >= a.n_items || *(volatile int *)a.error;
                if (!done && a.claim_ahead) claim = atomicAdd(a.head, (unsigned)chunk);  // in flight
                const int cnt = done ? 0 : min(chunk, a.n_items - base_i);
                BatchItem its[kChunk];
#pragma unroll
                for (int q = 0; q < kChunk; q++)
                    if (q < cnt) its[q] = a.items[base_i + q];
                for (int q = 0; q < cnt && !failed; q++)
                    if (!issue_item(&its[q], nullptr, 0xffffffffu)) failed = true;
                if (!failed && done && !issue_item(nullptr, nullptr, 0xffffffffu)) failed = true;
                if (failed || done) break;
                if (!a.claim_ahead) claim = atomicAdd(a.head, (unsigned)chunk);
            }
        }
        if (failed) {
            atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
            // no copy into this block's shared memory may still be in flight
            // when the block exits: wait (bounded) for the last loads issued
            for (int k = issued > ST ? issued - ST : 0; k < issued; k++)
                mbar_wait(&sh.full[k % ST], (k / ST) & 1, a.wait_limit_ns);
            // stop the compute warps and the storer after what was issued
            // (the stage is let drain first, bounded)
            const int s = issued % ST;
            if (issued >= ST) mbar_wait(&sh.empty[s], ((issued - ST) / ST) & 1, a.wait_limit_ns);
            sh.info[s].valid = 0;
            mbar_arrive(&sh.full[s]);
        }
        if (a.stats) {
            atomicAdd(a.stats + BS_DEP_WAIT, sh.st[BS_DEP_WAIT]);
            atomicAdd(a.stats + BS_REFILL_WAIT, sh.st[BS_REFILL_WAIT]);
            atomicAdd(a.stats + BS_PRODUCER_TOTAL, gtimer() - sh.st[BS_PRODUCER_TOTAL]);
            atomicAdd(a.stats + BS_ITEMS, (unsigned long long)issued);
            atomicAdd(a.stats + BS_BLOCKS, 1ull);
        }
        return;
    }

    if (warp == kStorerWarp) {
        // -------------------------------------------------------- storer
        if (threadIdx.x % 32 != 0) return;
        const int tile_px = kBatchTileElems;
        unsigned long long st_pub = 0;
        for (int j = 0;; j++) {
            const int s = j % ST;
            if (!mbar_wait(&sh.computed[s], (j / ST) & 1, a.wait_limit_ns)) {
                atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
                break;
            }
            const StageInfo inf = sh.info[s];
            if (!inf.valid) break;
            const float2 *stage = stages + (size_t)s * kStageElems;
            const unsigned char *tmaps = static_cast<const unsigned char *>(a.tmaps) +
                                         (size_t)inf.image * 128 * kBatchTmapsPerImage;
            if (inf.along_rows && inf.work) {
                // one 3-D box: the tile's rows into the column-tiled layout
                const int lines = tile_px / inf.cols;
                tensor3d_s2g(tmaps + 128, 0, 0, inf.tile * lines, stage);
            } else if (inf.along_rows) {
                const int n = inf.cols, lines = tile_px / n, row0 = inf.tile * lines;
                const int nrows = min(lines, inf.rows - row0);
                bulk_s2g(inf.dst + (size_t)row0 * n, stage, (unsigned)(nrows * n * sizeof(float2)));
            } else if (inf.ws_inplace && !inf.last) {
                // the columns block back in place in the workspace
                bulk_s2g(inf.work + (size_t)inf.tile * tile_px, stage,
                         (unsigned)(tile_px * sizeof(float2)));
            } else {
                const int n = inf.rows, w = tile_px / n, br = n < 256 ? n : 256;
                for (int b = 0; b < n / br; b++)
                    tensor2d_s2g(tmaps, inf.tile * w, b * br, stage + (size_t)b * br * w);
            }
            bulk_commit();
            const unsigned long long tw0 = a.stats ? gtimer() : 0;
            bulk_wait_read<0>();        // the stage may be refilled
            mbar_arrive(&sh.empty[s]);
            bulk_wait<0>();             // the tile is in global memory
            // the async-proxy writes are complete: order them before the release
            asm volatile("fence.proxy.async.global;" ::: "memory");
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            atomicAdd(a.done + inf.image * kBatchMaxPasses + inf.pass, 1u);
            if (a.stats) st_pub += gtimer() - tw0;
        }
        bulk_wait<0>();
        if (a.stats) atomicAdd(a.stats + BS_PUBLISH_WAIT, st_pub);
        return;
    }

    // ------------------------------------------------------------ compute
    const int tid = threadIdx.x;
    int cached_n = -1;
    if (a.stats && tid == 0) sh.st[BS_COMPUTE_TOTAL] = gtimer();
    for (int k = 0;; k++) {
        const int s = k % ST;
        const unsigned long long tf0 = (a.stats && tid == 0) ? gtimer() : 0;
        if (!mbar_wait(&sh.full[s], (k / ST) & 1, a.wait_limit_ns)) {
            if (tid == 0) atomicExch(a.error, GLSFFT_ERROR_TIMEOUT);
            break;
        }
        if (a.stats && tid == 0) sh.st[BS_FULL_WAIT] += gtimer() - tf0;
        const StageInfo in = sh.info[s];
        if (in.valid) ws_compute(stages + (size_t)s * kStageElems, in, a.tw, twc, tid, cached_n);
        // the generic-proxy writes of the results are ordered before the
        // storer's TMA store (and the next TMA write into the stage); the
        // stop record is passed on to the storer the same way
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&sh.computed[s]);
        if (!in.valid) break;
    }
    if (a.stats && tid == 0) {
        atomicAdd(a.stats + BS_FULL_WAIT, sh.st[BS_FULL_WAIT]);
        atomicAdd(a.stats + BS_COMPUTE_TOTAL, gtimer() - sh.st[BS_COMPUTE_TOTAL]);
    }
}

// Variants: blocks per SM -> (min blocks, stages): 1 -> (1, 3), 2 -> (2, 3),
// 3 -> (3, 2) (three blocks fit the SM's shared memory only with two stages).
template <int MINB, int ST>
static cudaError_t prepare_ws() {
    return smem_opt_in(reinterpret_cast<const void *>(fft_batch_ws<MINB, ST>), ws_smem<ST>());
}

template <int MINB, int ST>
static int ws_per_sm() {
    if (prepare_ws<MINB, ST>() != cudaSuccess) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fft_batch_ws<MINB, ST>, kBlock,
                                                      ws_smem<ST>()) != cudaSuccess)
        return 0;
    return per_sm;
}

cudaError_t launch_batch_ws(const BatchArgs &a, int grid, int blocks_per_sm, cudaStream_t s) {
    cudaError_t e = blocks_per_sm >= 3   ? prepare_ws<3, 2>()
                    : blocks_per_sm == 2 ? prepare_ws<2, 3>()
                                         : prepare_ws<1, 3>();
    if (e != cudaSuccess) return e;
    if (blocks_per_sm >= 3) fft_batch_ws<3, 2><<<grid, kBlock, ws_smem<2>(), s>>>(a);
    else if (blocks_per_sm == 2) fft_batch_ws<2, 3><<<grid, kBlock, ws_smem<3>(), s>>>(a);
    else fft_batch_ws<1, 3><<<grid, kBlock, ws_smem<3>(), s>>>(a);
    return cudaGetLastError();
}

int batch_ws_grid(int device, int blocks_per_sm) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return 0;
    int per_sm = blocks_per_sm >= 3 ? ws_per_sm<3, 2>() : blocks_per_sm == 2 ? ws_per_sm<2, 3>()
                                                                             : ws_per_sm<1, 3>();
    if (per_sm <= 0) return 0;
    if (per_sm > blocks_per_sm) per_sm = blocks_per_sm;
    return sms * per_sm;
}

}  // namespace glsfft
