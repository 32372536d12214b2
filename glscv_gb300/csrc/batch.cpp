// batch.cpp -- batch plans: uneven-size images, each run through one or two
// gls::fft transforms, executed as one CUDA graph.  Images the persistent
// kernels cover (16 <= rows <= 1024, 16 <= cols <= 4096, 16-byte aligned
// buffers) go through one persistent launch fed by a work list; any other
// image gets its own pass launches inside the same graph.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "batch_internal.h"
#include "batch_order.h"
#include "capi_internal.h"
#include "fft_config.h"
#include "glsfft_internal.h"

using namespace glsfft;

struct glsfft_batch_s {
    glsfft_context ctx = nullptr;
    int device = 0;
    int n_images = 0;      // images in the persistent launch
    int n_items = 0;
    int grid = 0;
    int variant = BATCH_TMA_WS3;   // the fastest variant measured on GB300
    void *d_mem = nullptr;  // tensor maps | images | passes | items | head, done, error
    void *d_work = nullptr;  // the images' column-tiled workspaces (BatchImage::work)
    BatchArgs args{};
    std::vector<BatchImage> images;
    std::vector<BatchPass> passes;
    struct Other {
        const void *src;
        void *dst;
        int rows, cols;
    };
    std::vector<Other> others;  // images outside the persistent kernels' shapes
    std::vector<int> flags;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long wait_limit_ns = 2000000000LL;
    size_t o_items = 0;
    int lag_items = 0;  // the item order's lag (order_items)
    unsigned long long *d_stats = nullptr;  // kBatchStats timing sums, when enabled
    struct Cand {
        int v, c, a, lg;
        double ms;
    };
    std::vector<Cand> tuned;  // the last autotuning's candidates
};

namespace {

// Default schedule: three warp-specialised blocks per SM, items claimed one
// at a time, an image's next pass listed five resident grids after its
// previous one -- the fastest schedule measured on GB300 for 64 x 1024^2
// forward + inverse (lag 4 is 0.5 % slower there and 2 % faster on 512
// uneven images, a difference the autotuner's 1 % keep margin lets it
// take), 7 % faster than two items per claim at a lag of eight grids
// (glsfft_batch_set_schedule / the autotuner can change all).
constexpr int kDefaultClaimChunk = 1;
constexpr int kDefaultLagGrids = 5;

int row_tiles_of(int rows, int cols) {
    const int lines = kBatchTileElems / cols;
    return (rows + lines - 1) / lines;
}
int col_tiles_of(int rows, int cols) {
    const int w = kBatchTileElems / rows;
    return (cols + w - 1) / w;
}

std::vector<BatchItem> order_items(const std::vector<BatchImage> &ims,
                                   const std::vector<BatchPass> &passes, int lag) {
    return order_work<BatchItem>(ims, passes, lag);
}

int grid_for(int device, int variant) {
    if (variant == BATCH_PLAIN) return batch_persistent_grid(device);
    return batch_ws_grid(device, variant);  // WS1..WS3: 1..3 blocks per SM
}

int record(glsfft_batch plan, cudaStream_t s) {
    if (plan->n_images > 0) {
        const size_t state = sizeof(unsigned) * (1 + (size_t)plan->n_images * kBatchMaxPasses) +
                             sizeof(int);
        cudaError_t e = cudaMemsetAsync(plan->args.head, 0, state, s);
        if (e != cudaSuccess) return cuda_status(e);
        if (plan->variant == BATCH_PLAIN)
            e = launch_batch_persistent(plan->args, plan->grid, s);
        else
            e = launch_batch_ws(plan->args, plan->grid, plan->variant, s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    for (const auto &o : plan->others) {
        const void *src = o.src;
        for (int f : plan->flags) {
            int st = fft2d_launch(plan->ctx, src, o.dst, o.rows, o.cols, f, false, s, 1);
            if (st) return st;
            src = o.dst;
        }
    }
    return GLSFFT_SUCCESS;
}

// (Re)capture the plan into a graph and instantiate it.
int capture(glsfft_batch plan) {
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    plan->exec = nullptr;
    plan->graph = nullptr;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(e);
    int st = GLSFFT_SUCCESS;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        st = cuda_status(e);
    } else {
        int rst = record(plan, cs);
        e = cudaStreamEndCapture(cs, &plan->graph);
        if (rst) st = rst;
        else if (e != cudaSuccess) st = cuda_status(e);
        if (!st) {
            e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
            if (e != cudaSuccess) st = cuda_status(e);
        }
    }
    cudaStreamDestroy(cs);
    cudaGetLastError();
    return st;
}

PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

}  // namespace

int glsfft::make_tmap_2d(void *tmap128, const void *base, long long width, long long height,
                         int box_w, int box_h) {
    auto enc = tmap_encoder();
    if (!enc) return GLSFFT_ERROR_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    cuuint64_t strides[1] = {(cuuint64_t)width * sizeof(float2)};
    cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(reinterpret_cast<CUtensorMap *>(tmap128), CU_TENSOR_MAP_DATA_TYPE_UINT64, 2,
                     const_cast<void *>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? GLSFFT_SUCCESS : GLSFFT_ERROR_CUDA;
}

int glsfft::make_column_tmap(void *tmap128, const void *img, int rows, int cols) {
    const int w = kBatchTileElems / rows;     // columns per tile
    const int br = rows < 256 ? rows : 256;   // box height (TMA box dims <= 256)
    return make_tmap_2d(tmap128, img, cols, rows, w, br);
}

int glsfft::make_tiled_tmap(void *tmap128, const void *work, int rows, int cols, bool swizzled) {
    if (!batch_tiled_ok(rows, cols)) return GLSFFT_ERROR_INVALID_VALUE;
    auto enc = tmap_encoder();
    if (!enc) return GLSFFT_ERROR_CUDA;
    const int w = kBatchTileElems / rows, lines = kBatchTileElems / cols;
    if (swizzled) {
        if (!batch_tiled_inplace(rows, cols)) return GLSFFT_ERROR_INVALID_VALUE;
        cuuint64_t d2[2] = {(cuuint64_t)rows * w, (cuuint64_t)(cols / w)};
        cuuint64_t s2[1] = {(cuuint64_t)rows * w * sizeof(float2)};
        cuuint32_t b2[2] = {(cuuint32_t)(lines * w), (cuuint32_t)(cols / w)};
        cuuint32_t e2[2] = {1, 1};
        CUresult r2 = enc(reinterpret_cast<CUtensorMap *>(tmap128), CU_TENSOR_MAP_DATA_TYPE_UINT64,
                          2, const_cast<void *>(work), d2, s2, b2, e2, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        return r2 == CUDA_SUCCESS ? GLSFFT_SUCCESS : GLSFFT_ERROR_CUDA;
    }
    cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)(cols / w), (cuuint64_t)rows};
    cuuint64_t strides[2] = {(cuuint64_t)rows * w * sizeof(float2), (cuuint64_t)w * sizeof(float2)};
    cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)(cols / w), (cuuint32_t)lines};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(reinterpret_cast<CUtensorMap *>(tmap128), CU_TENSOR_MAP_DATA_TYPE_UINT64, 3,
                     const_cast<void *>(work), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? GLSFFT_SUCCESS : GLSFFT_ERROR_CUDA;
}

extern "C" {

int glsfft_batch_create(glsfft_context ctx, int count, const void *const *srcs,
                        void *const *dsts, const int *rows, const int *cols, int n_transforms,
                        const int *flags, glsfft_batch *out) {
    if (!out) return GLSFFT_ERROR_INVALID_VALUE;
    *out = nullptr;
    if (!srcs || !dsts || !rows || !cols || !flags || count < 1) return GLSFFT_ERROR_INVALID_VALUE;
    if (n_transforms < 1 || n_transforms > kBatchMaxPasses / 2) return GLSFFT_ERROR_INVALID_VALUE;
    for (int k = 0; k < n_transforms; k++) {
        if (flags[k] & ~(GLSFFT_INVERSE | GLSFFT_SCALE | GLSFFT_SHIFT))
            return GLSFFT_ERROR_INVALID_VALUE;
    }
    for (int i = 0; i < count; i++) {
        int st = check_fft_args(srcs[i], dsts[i], rows[i], cols[i], 0, false);
        if (st) return st;
    }
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;

    auto *plan = new (std::nothrow) glsfft_batch_s();
    if (!plan) return GLSFFT_ERROR_OUT_OF_MEMORY;
    plan->ctx = ctx;
    plan->device = ctx->device;
    plan->flags.assign(flags, flags + n_transforms);

    // the pass chain: rows then columns per transform, gls::fft's flags split
    // per pass exactly as glsfft_fft2d_c2c does for a 2-D image
    for (int k = 0; k < n_transforms; k++) {
        const bool inv = flags[k] & GLSFFT_INVERSE, sc = flags[k] & GLSFFT_SCALE,
                   sh = flags[k] & GLSFFT_SHIFT;
        plan->passes.push_back(BatchPass{1, (inv ? PF_CONJ_IN : 0u) | (sh ? PF_SHIFT_COLS : 0u), sc, 0});
        plan->passes.push_back(BatchPass{0, (inv ? PF_CONJ_OUT : 0u) | (sh ? PF_SHIFT_ROWS : 0u), sc, 0});
    }

    for (int i = 0; i < count; i++) {
        const bool aligned16 = ((reinterpret_cast<uintptr_t>(srcs[i]) |
                                 reinterpret_cast<uintptr_t>(dsts[i])) & 15) == 0;
        if (batch_supported(rows[i], cols[i]) && aligned16) {
            BatchImage im{};
            im.src = static_cast<const float2 *>(srcs[i]);
            im.dst = static_cast<float2 *>(dsts[i]);
            im.rows = rows[i];
            im.cols = cols[i];
            im.row_tiles = row_tiles_of(rows[i], cols[i]);
            im.col_tiles = col_tiles_of(rows[i], cols[i]);
            plan->images.push_back(im);
        } else {
            plan->others.push_back({srcs[i], dsts[i], rows[i], cols[i]});
        }
    }
    plan->n_images = (int)plan->images.size();
    int st = GLSFFT_SUCCESS;
    if (plan->n_images > 0) {
        plan->grid = grid_for(ctx->device, plan->variant);
        if (plan->grid <= 0) st = GLSFFT_ERROR_CUDA;
        std::vector<BatchItem> items;
        plan->lag_items = kDefaultLagGrids * plan->grid;
        if (!st) items = order_items(plan->images, plan->passes, plan->lag_items);
        plan->n_items = (int)items.size();
        const size_t ni = plan->images.size();
        const size_t b_tm = 128 * kBatchTmapsPerImage * ni;
        const size_t b_im = sizeof(BatchImage) * ni;
        const size_t b_ps = sizeof(BatchPass) * plan->passes.size();
        const size_t b_it = sizeof(BatchItem) * items.size();
        const size_t b_state = sizeof(unsigned) * (1 + ni * kBatchMaxPasses) + sizeof(int);
        auto up = [](size_t x) { return (x + 255) / 256 * 256; };
        const size_t o_im = up(b_tm), o_ps = o_im + up(b_im), o_it = o_ps + up(b_ps),
                     o_st = o_it + up(b_it), total = o_st + b_state;
        plan->o_items = o_it;
        if (!st && ctx->budget && total > ctx->budget) st = GLSFFT_ERROR_BUDGET;
        if (!st && cudaMalloc(&plan->d_mem, total) != cudaSuccess) {
            cudaGetLastError();
            st = GLSFFT_ERROR_OUT_OF_MEMORY;
        }
        // Column-tiled workspaces (one image each, 256-byte aligned) for
        // the images whose shape allows them, when they fit the context's
        // budget next to the plan's tables; otherwise the columns passes
        // read and write dst in place through the column map.
        size_t b_work = 0;
        for (const BatchImage &im : plan->images)
            if (batch_tiled_ok(im.rows, im.cols))
                b_work += up(sizeof(float2) * (size_t)im.rows * im.cols);
        if (!st && b_work && (!ctx->budget || total + b_work <= ctx->budget) &&
            cudaMalloc(&plan->d_work, b_work) != cudaSuccess) {
            cudaGetLastError();
            plan->d_work = nullptr;
        }
        if (plan->d_work) {
            char *w = static_cast<char *>(plan->d_work);
            for (BatchImage &im : plan->images) {
                if (!batch_tiled_ok(im.rows, im.cols)) continue;
                im.work = reinterpret_cast<float2 *>(w);
                im.ws_inplace = batch_tiled_inplace(im.rows, im.cols) ? 1 : 0;
                w += up(sizeof(float2) * (size_t)im.rows * im.cols);
            }
        }
        if (!st) {
            std::vector<unsigned char> host(o_st, 0);
            for (size_t i = 0; i < ni && !st; i++) {
                BatchImage &im = plan->images[i];
                unsigned char *tm = host.data() + 128 * kBatchTmapsPerImage * i;
                st = make_column_tmap(tm, im.dst, im.rows, im.cols);
                // an encoder that refuses the tiled map leaves the image in place
                if (!st && im.work &&
                    (make_tiled_tmap(tm + 128, im.work, im.rows, im.cols, false) ||
                     (im.ws_inplace && make_tiled_tmap(tm + 256, im.work, im.rows, im.cols, true)))) {
                    im.work = nullptr;
                    im.ws_inplace = 0;
                }
            }
            std::memcpy(host.data() + o_im, plan->images.data(), b_im);
            std::memcpy(host.data() + o_ps, plan->passes.data(), b_ps);
            std::memcpy(host.data() + o_it, items.data(), b_it);
            char *base = static_cast<char *>(plan->d_mem);
            if (!st) {
                cudaError_t e = cudaMemcpy(base, host.data(), o_st, cudaMemcpyHostToDevice);
                if (e != cudaSuccess) st = cuda_status(e);
            }
            BatchArgs &a = plan->args;
            a.tmaps = base;
            a.images = reinterpret_cast<const BatchImage *>(base + o_im);
            a.passes = reinterpret_cast<const BatchPass *>(base + o_ps);
            a.items = reinterpret_cast<const BatchItem *>(base + o_it);
            a.n_items = plan->n_items;
            a.n_passes = (int)plan->passes.size();
            a.head = reinterpret_cast<unsigned *>(base + o_st);
            a.done = a.head + 1;
            a.error = reinterpret_cast<int *>(a.done + ni * kBatchMaxPasses);
            a.tw = ctx->d_tw;
            a.wait_limit_ns = plan->wait_limit_ns;
            a.claim_chunk = kDefaultClaimChunk;
            a.claim_ahead = 0;
        }
    }
    if (!st) st = capture(plan);
    if (st) {
        if (plan->exec) cudaGraphExecDestroy(plan->exec);
        if (plan->graph) cudaGraphDestroy(plan->graph);
        if (plan->d_mem) cudaFree(plan->d_mem);
        if (plan->d_work) cudaFree(plan->d_work);
        delete plan;
        return st;
    }
    *out = plan;
    return GLSFFT_SUCCESS;
}

int glsfft_batch_set_variant(glsfft_batch plan, int variant) {
    if (!plan || variant < BATCH_PLAIN || variant > BATCH_TMA_WS3) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    if (plan->n_images > 0) {
        const int grid = grid_for(plan->device, variant);
        if (grid <= 0) return GLSFFT_ERROR_CUDA;
        if (grid != plan->grid) {
            // the item order's lag follows the resident grid
            std::vector<BatchItem> items =
                order_items(plan->images, plan->passes, kDefaultLagGrids * grid);
            cudaError_t e = cudaMemcpy(static_cast<char *>(plan->d_mem) + plan->o_items,
                                       items.data(), sizeof(BatchItem) * items.size(),
                                       cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cuda_status(e);
            plan->grid = grid;
            plan->lag_items = kDefaultLagGrids * grid;
        }
    }
    plan->variant = variant;
    return capture(plan);
}

int glsfft_batch_set_schedule(glsfft_batch plan, int claim_chunk, int claim_ahead, int lag_blocks) {
    if (!plan || claim_chunk < 1 || claim_chunk > 4 || lag_blocks < 0)
        return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    plan->args.claim_chunk = claim_chunk;
    plan->args.claim_ahead = claim_ahead < 0 ? 0 : (claim_ahead > 2 ? 2 : claim_ahead);
    if (plan->n_images > 0 && lag_blocks > 0) {
        std::vector<BatchItem> items = order_items(plan->images, plan->passes, lag_blocks);
        cudaError_t e = cudaMemcpy(static_cast<char *>(plan->d_mem) + plan->o_items, items.data(),
                                   sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_status(e);
        plan->lag_items = lag_blocks;
    }
    return capture(plan);
}

int glsfft_batch_execute(glsfft_batch plan, void *stream) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    return cuda_status(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
}

int glsfft_batch_status(glsfft_batch plan, void *stream) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    if (plan->n_images == 0) return GLSFFT_SUCCESS;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, plan->args.error, sizeof(int), cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_status(e);
    return err;
}

int glsfft_batch_info(glsfft_batch plan, int *persistent_images, int *items, int *grid) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    if (persistent_images) *persistent_images = plan->n_images;
    if (items) *items = plan->n_items;
    if (grid) *grid = plan->grid;
    return GLSFFT_SUCCESS;
}

int glsfft_batch_workspace(glsfft_batch plan, int *tiled_images, size_t *bytes) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    int n = 0;
    size_t b = 0;
    for (const BatchImage &im : plan->images) {
        if (!im.work) continue;
        n++;
        b += (sizeof(float2) * (size_t)im.rows * im.cols + 255) / 256 * 256;
    }
    if (tiled_images) *tiled_images = n;
    if (bytes) *bytes = b;
    return GLSFFT_SUCCESS;
}

int glsfft_batch_inject_stall(glsfft_batch plan, long long wait_limit_ns) {
    // host-side fault injection: the last item of the list waits for one more
    // tile than its previous pass has, so its bounded wait must expire
    if (!plan || plan->n_images == 0 || plan->n_items < 1 || wait_limit_ns <= 0)
        return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    BatchItem last{};
    const BatchItem *d_last = plan->args.items + plan->n_items - 1;
    cudaError_t e = cudaMemcpy(&last, d_last, sizeof(last), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    if (last.pass == 0) return GLSFFT_ERROR_INVALID_VALUE;
    last.need += 1;
    e = cudaMemcpy(const_cast<BatchItem *>(d_last), &last, sizeof(last), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
    // the deadline is a kernel argument baked into the graph: re-capture
    plan->wait_limit_ns = wait_limit_ns;
    plan->args.wait_limit_ns = wait_limit_ns;
    return capture(plan);
}

int glsfft_batch_get_schedule(glsfft_batch plan, int *out4) {
    if (!plan || !out4) return GLSFFT_ERROR_INVALID_VALUE;
    out4[0] = plan->variant;
    out4[1] = plan->args.claim_chunk ? plan->args.claim_chunk : kDefaultClaimChunk;
    out4[2] = plan->args.claim_ahead;
    out4[3] = plan->lag_items;
    return GLSFFT_SUCCESS;
}

int glsfft_batch_autotune(glsfft_batch plan, const char *cache_path, int reps, void *stream,
                          int *result, double *ms) {
    if (!plan || reps < 1 || reps > 1000) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    glsfft_context ctx = plan->ctx;
    cudaStream_t s = (cudaStream_t)stream;
    int st = GLSFFT_SUCCESS;

    // 1. per-size pass schedules of the images that get their own launches
    std::map<std::pair<int, int>, int> other_sizes;
    for (const auto &o : plan->others) other_sizes[{o.rows, o.cols}]++;
    for (const auto &kv : other_sizes) {
        st = glsfft_autotune_fft2d(ctx, kv.first.first, kv.first.second,
                                   std::min(kv.second, 64), cache_path, stream, nullptr, nullptr);
        if (st) return st;
    }

    int res[6] = {plan->variant, plan->args.claim_chunk, plan->args.claim_ahead, plan->lag_items,
                  0, 0};
    double t[2] = {0.0, 0.0};
    if (plan->n_images == 0) {  // nothing persistent: re-record the per-size schedules
        st = capture(plan);
        if (!st && result) std::copy(res, res + 6, result);
        if (!st && ms) std::copy(t, t + 2, ms);
        return st;
    }

    // 2. the plan key: device, the persistent images' and the other images'
    //    size histograms, the transform flags
    auto histogram = [](const std::map<std::pair<int, int>, int> &h) {
        std::string o;
        for (const auto &kv : h) {
            if (!o.empty()) o += ";";
            o += std::to_string(kv.first.first) + "x" + std::to_string(kv.first.second) + "*" +
                 std::to_string(kv.second);
        }
        return o;
    };
    std::map<std::pair<int, int>, int> pers;
    for (const auto &im : plan->images) pers[{im.rows, im.cols}]++;
    std::string flags;
    for (int f : plan->flags) flags += (flags.empty() ? "" : ",") + std::to_string(f);
    plan_cache::Pairs key = device_fields(plan->device);
    key.push_back({"kind", plan_cache::quote("batch")});
    key.push_back({"persistent", plan_cache::quote(histogram(pers))});
    key.push_back({"others", plan_cache::quote(histogram(other_sizes))});
    key.push_back({"flags", plan_cache::quote(flags)});

    auto apply = [&](int variant, int chunk, int ahead, int lag_grids) {
        int r = glsfft_batch_set_variant(plan, variant);
        if (!r) r = glsfft_batch_set_schedule(plan, chunk, ahead, lag_grids * plan->grid);
        return r;
    };
    plan_cache::Fields hit;
    if (plan_cache::lookup(cache_path, plan_cache::as_fields(key), hit)) {
        const int v = std::atoi(hit["variant"].c_str()), c = std::atoi(hit["claim_chunk"].c_str()),
                  a = std::atoi(hit["claim_ahead"].c_str()),
                  lg = std::atoi(hit["lag_grids"].c_str());
        if (v >= BATCH_PLAIN && v <= BATCH_TMA_WS3 && c >= 1 && c <= 4 && a >= 0 && a <= 2 &&
            lg >= 1) {
            st = apply(v, c, a, lg);
            if (st) return st;
            res[0] = v;
            res[1] = c;
            res[2] = a;
            res[3] = plan->lag_items;
            res[4] = 1;
            t[0] = std::atof(hit["ms"].c_str());
            t[1] = std::atof(hit["ms_default"].c_str());
            if (result) std::copy(res, res + 6, result);
            if (ms) std::copy(t, t + 2, ms);
            return GLSFFT_SUCCESS;
        }
    }

    // 3. a shadow plan of the same shapes, flags, pointer alignments and
    //    src/dst aliasing on scratch buffers: the caller's images are not touched
    struct Shadow {
        int rows, cols;
        uintptr_t src_off, dst_off;
        bool alias;
        size_t src_at, dst_at;
    };
    std::vector<Shadow> sh;
    size_t total = 0;
    auto take = [&](size_t bytes) {
        const size_t at = total;
        total += (bytes + 16 + 255) / 256 * 256;
        return at;
    };
    auto add = [&](const void *src, const void *dst, int rows, int cols) {
        Shadow x{rows, cols, reinterpret_cast<uintptr_t>(src) & 15,
                 reinterpret_cast<uintptr_t>(dst) & 15, src == dst, 0, 0};
        const size_t bytes = (size_t)rows * cols * sizeof(float2);
        x.src_at = take(bytes);
        x.dst_at = x.alias ? x.src_at : take(bytes);
        sh.push_back(x);
    };
    for (const auto &im : plan->images) add(im.src, im.dst, im.rows, im.cols);
    for (const auto &o : plan->others) add(o.src, o.dst, o.rows, o.cols);
    if (ctx->budget && total > ctx->budget) return GLSFFT_ERROR_BUDGET;
    char *scratch = nullptr;
    cudaError_t e = cudaMalloc(&scratch, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GLSFFT_ERROR_OUT_OF_MEMORY;
    }
    e = cudaMemsetAsync(scratch, 0x3f, total, s);  // finite values
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e);
    std::vector<const void *> ssrc;
    std::vector<void *> sdst;
    std::vector<int> srows, scols;
    for (const auto &x : sh) {
        ssrc.push_back(scratch + x.src_at + x.src_off);
        sdst.push_back(scratch + x.dst_at + x.dst_off);
        srows.push_back(x.rows);
        scols.push_back(x.cols);
    }
    glsfft_batch shadow = nullptr;
    if (!st)
        st = glsfft_batch_create(ctx, (int)sh.size(), ssrc.data(), sdst.data(), srows.data(),
                                 scols.data(), (int)plan->flags.size(), plan->flags.data(),
                                 &shadow);
    if (!st && shadow->n_images != plan->n_images) st = GLSFFT_ERROR_CUDA;  // routing differs

    // 4. every schedule: variant x item-order lag (resident grids) x claim
    //    chunk x claim-ahead (the plain variant has no claim knobs)
    using Cand = glsfft_batch_s::Cand;
    std::vector<Cand> cands;
    const int variants[4] = {BATCH_TMA_WS2, BATCH_TMA_WS3, BATCH_TMA_WS1, BATCH_PLAIN};
    const int lags[6] = {2, 3, 4, 5, 6, 8};
    for (int v : variants) {
        for (int lg : lags) {
            for (int c = 1; c <= 4 && !st; c *= 2) {
                if (v == BATCH_PLAIN && c != kDefaultClaimChunk) continue;
                for (int a = 0; a <= 2 && !st; a++) {
                    if (v == BATCH_PLAIN && a) continue;
                    if (a == 2 && c != 1) continue;  // deep prefetch claims one item at a time
                    st = glsfft_batch_set_variant(shadow, v);
                    if (!st) st = glsfft_batch_set_schedule(shadow, c, a, lg * shadow->grid);
                    double m = 0.0;
                    if (!st)
                        st = time_median_ms([&]() { return glsfft_batch_execute(shadow, s); }, 2,
                                            reps, s, &m);
                    if (!st) {
                        const int dev_st = glsfft_batch_status(shadow, s);
                        if (dev_st == GLSFFT_ERROR_TIMEOUT) continue;  // not a usable schedule
                        st = dev_st;
                    }
                    if (!st) cands.push_back(Cand{v, c, a, lg, m});
                }
            }
        }
    }
    auto is_default = [](const Cand &c) {
        return c.v == BATCH_TMA_WS3 && c.c == kDefaultClaimChunk && c.a == 0 &&
               c.lg == kDefaultLagGrids;
    };
    // 5. the finalists -- the six fastest of that sweep and the default --
    //    timed again in three interleaved rounds; each keeps the median of its
    //    three medians, so one noisy sample does not pick the schedule
    std::vector<size_t> finalists;
    if (!st && !cands.empty()) {
        std::vector<size_t> order(cands.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = i;
        std::sort(order.begin(), order.end(),
                  [&](size_t x, size_t y) { return cands[x].ms < cands[y].ms; });
        finalists.assign(order.begin(), order.begin() + std::min<size_t>(6, order.size()));
        for (size_t i = 0; i < cands.size(); i++)
            if (is_default(cands[i]) &&
                std::find(finalists.begin(), finalists.end(), i) == finalists.end())
                finalists.push_back(i);
        std::vector<std::vector<double>> runs(finalists.size());
        for (int r = 0; r < 3 && !st; r++) {
            for (size_t j = 0; j < finalists.size() && !st; j++) {
                const Cand &c = cands[finalists[j]];
                st = glsfft_batch_set_variant(shadow, c.v);
                if (!st) st = glsfft_batch_set_schedule(shadow, c.c, c.a, c.lg * shadow->grid);
                double m = 0.0;
                if (!st)
                    st = time_median_ms([&]() { return glsfft_batch_execute(shadow, s); }, 1,
                                        reps, s, &m);
                if (!st) runs[j].push_back(m);
            }
        }
        if (!st) st = glsfft_batch_status(shadow, s);
        if (!st) {
            for (size_t j = 0; j < finalists.size(); j++) {
                std::sort(runs[j].begin(), runs[j].end());
                cands[finalists[j]].ms = runs[j][1];
            }
        }
    }
    if (shadow) glsfft_batch_destroy(shadow);
    cudaStreamSynchronize(s);
    cudaFree(scratch);
    cudaGetLastError();
    if (st) return st;
    if (cands.empty()) return GLSFFT_ERROR_TIMEOUT;
    plan->tuned = cands;

    // 6. the fastest finalist, unless the default schedule is within the keep
    //    margin
    const Cand *best = &cands[finalists[0]], *def = nullptr;
    for (size_t i : finalists) {
        const Cand &c = cands[i];
        if (c.ms < best->ms) best = &c;
        if (is_default(c)) def = &c;
    }
    if (def && best->ms > def->ms * 0.99) best = def;
    st = apply(best->v, best->c, best->a, best->lg);
    if (st) return st;
    res[0] = best->v;
    res[1] = best->c;
    res[2] = best->a;
    res[3] = plan->lag_items;
    res[5] = (int)cands.size();
    t[0] = best->ms;
    t[1] = def ? def->ms : 0.0;
    if (cache_path && *cache_path) {
        key.push_back({"variant", std::to_string(best->v)});
        key.push_back({"claim_chunk", std::to_string(best->c)});
        key.push_back({"claim_ahead", std::to_string(best->a)});
        key.push_back({"lag_grids", std::to_string(best->lg)});
        char b[64];
        std::snprintf(b, sizeof b, "%.6g", t[0]);
        key.push_back({"ms", b});
        std::snprintf(b, sizeof b, "%.6g", t[1]);
        key.push_back({"ms_default", b});
        key.push_back({"candidates", std::to_string(cands.size())});
        if (!plan_cache::append(cache_path, key)) st = GLSFFT_ERROR_IO;
    }
    if (result) std::copy(res, res + 6, result);
    if (ms) std::copy(t, t + 2, ms);
    return st;
}

int glsfft_batch_set_stats(glsfft_batch plan, int on) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    if (on && !plan->d_stats) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(unsigned long long) * kBatchStats) != cudaSuccess) {
            cudaGetLastError();
            return GLSFFT_ERROR_OUT_OF_MEMORY;
        }
        cudaError_t e = cudaMemset(p, 0, sizeof(unsigned long long) * kBatchStats);
        if (e != cudaSuccess) {
            cudaFree(p);
            return cuda_status(e);
        }
        plan->d_stats = static_cast<unsigned long long *>(p);
    }
    plan->args.stats = on ? plan->d_stats : nullptr;
    return capture(plan);
}

int glsfft_batch_get_stats(glsfft_batch plan, void *stream, double *out) {
    if (!plan || !out) return GLSFFT_ERROR_INVALID_VALUE;
    for (int i = 0; i < kBatchStats; i++) out[i] = 0.0;
    if (!plan->d_stats) return GLSFFT_SUCCESS;
    DeviceGuard g(plan->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    unsigned long long h[kBatchStats];
    cudaError_t e = cudaMemcpyAsync(h, plan->d_stats, sizeof h, cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(plan->d_stats, 0, sizeof h, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_status(e);
    for (int i = 0; i < kBatchStats; i++) out[i] = (double)h[i];
    return GLSFFT_SUCCESS;
}

int glsfft_batch_tuning(glsfft_batch plan, int max, int *sched4, double *ms, int *count) {
    if (!plan || !count || max < 0 || (max > 0 && (!sched4 || !ms)))
        return GLSFFT_ERROR_INVALID_VALUE;
    *count = (int)plan->tuned.size();
    for (int i = 0; i < max && i < (int)plan->tuned.size(); i++) {
        const auto &c = plan->tuned[i];
        sched4[4 * i] = c.v;
        sched4[4 * i + 1] = c.c;
        sched4[4 * i + 2] = c.a;
        sched4[4 * i + 3] = c.lg;
        ms[i] = c.ms;
    }
    return GLSFFT_SUCCESS;
}

int glsfft_batch_destroy(glsfft_batch plan) {
    if (!plan) return GLSFFT_ERROR_INVALID_VALUE;
    DeviceGuard g(plan->device);
    if (plan->d_stats) cudaFree(plan->d_stats);
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    if (plan->d_mem) cudaFree(plan->d_mem);
    if (plan->d_work) cudaFree(plan->d_work);
    delete plan;
    return GLSFFT_SUCCESS;
}

}  // extern "C"
