// transfer.cpp -- gls::fft over images in host memory with the transfers
// pipelined against the transforms (the GlsMat upload / download path,
// glsCV/glsMat.cpp:374-417 and :493-551, made asynchronous and overlapped).
//
// The images are cut into chunks.  Chunk k is copied host -> device into
// slot k % kSlots of a ring of device buffers on the "up" stream, transformed
// there by the slot's batch plan on the "compute" stream, and copied back on
// the "down" stream; events order the three, so while chunk k is being
// transformed chunk k+1 is arriving and chunk k-1 is leaving.  A slot is
// refilled only after its previous chunk has left.  The ring, the streams
// and the plans are kept in the context and rebuilt when the shape, chunk
// or flags change.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

#include "capi_internal.h"
#include "glsfft.h"

using namespace glsfft;

namespace {

constexpr int kSlots = 3;
constexpr size_t kAutoChunkBytes = 32u << 20;  // automatic chunk: about 32 MiB of images

}  // namespace

struct HostPipe {
    int rows = 0, cols = 0, chunk = 0;
    std::vector<int> flags;
    cudaStream_t up = nullptr, compute = nullptr, down = nullptr;
    cudaEvent_t start = nullptr;
    cudaEvent_t uploaded[kSlots] = {}, computed[kSlots] = {}, downloaded[kSlots] = {};
    bool used[kSlots] = {};
    void *slot[kSlots] = {};
    glsfft_batch plan[kSlots] = {};
};

void glsfft::host_pipe_destroy(HostPipe *p) {
    if (!p) return;
    if (p->up) cudaStreamSynchronize(p->up);
    if (p->compute) cudaStreamSynchronize(p->compute);
    if (p->down) cudaStreamSynchronize(p->down);
    for (int i = 0; i < kSlots; i++) {
        if (p->plan[i]) glsfft_batch_destroy(p->plan[i]);
        if (p->slot[i]) cudaFree(p->slot[i]);
        if (p->uploaded[i]) cudaEventDestroy(p->uploaded[i]);
        if (p->computed[i]) cudaEventDestroy(p->computed[i]);
        if (p->downloaded[i]) cudaEventDestroy(p->downloaded[i]);
    }
    if (p->start) cudaEventDestroy(p->start);
    if (p->up) cudaStreamDestroy(p->up);
    if (p->compute) cudaStreamDestroy(p->compute);
    if (p->down) cudaStreamDestroy(p->down);
    cudaGetLastError();
    delete p;
}

namespace {

// The context's pipeline for this shape, chunk and flag chain (built once).
int get_pipe(glsfft_context ctx, int rows, int cols, int chunk, const int *flags, int nt,
             HostPipe **out) {
    HostPipe *p = ctx->host_pipe;
    if (p && p->rows == rows && p->cols == cols && p->chunk == chunk &&
        p->flags == std::vector<int>(flags, flags + nt)) {
        *out = p;
        return GLSFFT_SUCCESS;
    }
    host_pipe_destroy(p);
    ctx->host_pipe = nullptr;
    const size_t img = (size_t)rows * cols * sizeof(float2);
    const size_t slot_bytes = img * (size_t)chunk;
    if (ctx->budget && slot_bytes * kSlots > ctx->budget) return GLSFFT_ERROR_BUDGET;
    p = new (std::nothrow) HostPipe();
    if (!p) return GLSFFT_ERROR_OUT_OF_MEMORY;
    p->rows = rows;
    p->cols = cols;
    p->chunk = chunk;
    p->flags.assign(flags, flags + nt);
    cudaError_t e = cudaStreamCreateWithFlags(&p->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->compute, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->down, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->start, cudaEventDisableTiming);
    for (int i = 0; i < kSlots && e == cudaSuccess; i++) {
        e = cudaEventCreateWithFlags(&p->uploaded[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->computed[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->downloaded[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&p->slot[i], slot_bytes);
    }
    int st = cuda_status(e);
    // one batch plan per slot, transforming the slot's images in place
    std::vector<const void *> srcs(chunk);
    std::vector<void *> dsts(chunk);
    std::vector<int> rs(chunk, rows), cs(chunk, cols);
    for (int i = 0; i < kSlots && !st; i++) {
        for (int j = 0; j < chunk; j++) {
            dsts[j] = static_cast<char *>(p->slot[i]) + img * j;
            srcs[j] = dsts[j];
        }
        st = glsfft_batch_create(ctx, chunk, srcs.data(), dsts.data(), rs.data(), cs.data(), nt,
                                 flags, &p->plan[i]);
    }
    if (st) {
        cudaGetLastError();
        host_pipe_destroy(p);
        return st;
    }
    ctx->host_pipe = p;
    *out = p;
    return GLSFFT_SUCCESS;
}

}  // namespace

extern "C" {

int glsfft_fft2d_host(glsfft_context ctx, const void *host_src, void *host_dst, int count,
                      int rows, int cols, int n_transforms, const int *flags, int chunk,
                      void *stream) {
    if (!ctx || !host_src || !host_dst || !flags || count < 1 || chunk < 0)
        return GLSFFT_ERROR_INVALID_VALUE;
    if (n_transforms < 1 || n_transforms > 2) return GLSFFT_ERROR_INVALID_VALUE;
    for (int k = 0; k < n_transforms; k++)
        if (flags[k] & ~(GLSFFT_INVERSE | GLSFFT_SCALE | GLSFFT_SHIFT))
            return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    if (((reinterpret_cast<uintptr_t>(host_src) | reinterpret_cast<uintptr_t>(host_dst)) & 7) != 0)
        return GLSFFT_ERROR_MISALIGNED;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;

    const size_t img = (size_t)rows * cols * sizeof(float2);
    if (chunk == 0) {
        // about 32 MiB per chunk, and at least four chunks when there are
        // enough images for the copies to overlap the transforms
        const size_t by_bytes = std::max<size_t>(1, kAutoChunkBytes / img);
        const size_t quarter = (size_t)(count + 3) / 4;
        chunk = (int)std::max<size_t>(1, std::min(by_bytes, quarter));
    }
    chunk = std::min(chunk, std::min(count, kMaxBatch));
    HostPipe *p = nullptr;
    st = get_pipe(ctx, rows, cols, chunk, flags, n_transforms, &p);
    if (st) return st;

    cudaStream_t user = (cudaStream_t)stream;
    // everything after the work already queued on the caller's stream
    cudaError_t e = cudaEventRecord(p->start, user);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->up, p->start, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(p->down, p->start, 0);
    const char *src = static_cast<const char *>(host_src);
    char *dst = static_cast<char *>(host_dst);
    const int chunks = (count + chunk - 1) / chunk;
    int last = 0;
    for (int k = 0; k < chunks && e == cudaSuccess && !st; k++) {
        const int i = k % kSlots, n = std::min(chunk, count - k * chunk);
        const size_t off = img * (size_t)chunk * k, bytes = img * (size_t)n;
        // up: the slot's previous chunk must have left
        if (p->used[i]) e = cudaStreamWaitEvent(p->up, p->downloaded[i], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->slot[i], src + off, bytes, cudaMemcpyHostToDevice, p->up);
        if (e == cudaSuccess) e = cudaEventRecord(p->uploaded[i], p->up);
        // compute: the slot's plan, or batched pass launches for a short tail
        if (e == cudaSuccess) e = cudaStreamWaitEvent(p->compute, p->uploaded[i], 0);
        if (e == cudaSuccess) {
            if (n == chunk) {
                st = glsfft_batch_execute(p->plan[i], p->compute);
            } else {
                for (int t = 0; t < n_transforms && !st; t++)
                    st = fft2d_launch(ctx, p->slot[i], p->slot[i], rows, cols, flags[t], false,
                                      p->compute, n);
            }
        }
        if (e == cudaSuccess && !st) e = cudaEventRecord(p->computed[i], p->compute);
        // down
        if (e == cudaSuccess && !st) e = cudaStreamWaitEvent(p->down, p->computed[i], 0);
        if (e == cudaSuccess && !st)
            e = cudaMemcpyAsync(dst + off, p->slot[i], bytes, cudaMemcpyDeviceToHost, p->down);
        if (e == cudaSuccess && !st) e = cudaEventRecord(p->downloaded[i], p->down);
        p->used[i] = true;
        last = i;
    }
    // the caller's stream continues after the last chunk has left
    if (e == cudaSuccess && !st) e = cudaStreamWaitEvent(user, p->downloaded[last], 0);
    if (st) return st;
    return cuda_status(e);
}

}  // extern "C"
