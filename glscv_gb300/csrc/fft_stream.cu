// fft_stream.cu -- the streamed column pass for 2048- and 4096-point columns
// (pass schedule kSchedStreamed).
//
// A tile of the plain column kernel for 4096-point columns (4 columns, 32
// bytes of each image row: the narrowest segment that keeps whole DRAM
// sectors) is 128 KB, so an SM holds one tile at a time and loads,
// transforms and stores it in turn: HBM idles while the SM computes.  Here
// one persistent 1024-thread block per SM walks the column tiles of the
// batch (image-major, then tile) and keeps the NEXT tile's copy in flight
// while it transforms the current one:
//   * the tile (L columns x N rows, L * N * 8 = 128 KB) lands in a
//     shared-memory stage as N/256 2-D tensor boxes of L x 256 (Tensor Memory
//     Accelerator, one tensor map over the whole batch), completing on an
//     mbarrier;
//   * every thread copies its 16 values of one column to registers, the
//     block syncs, and thread 0 at once issues the next tile's copy;
//   * the Stockham passes exchange through a separate float buffer, real and
//     imaginary parts in turn (half the shared memory of a complex exchange,
//     so stage + exchange fit one SM: 128 KB + 68 KB);
//   * results are stored from registers as whole 32- (N = 4096) or 64-byte
//     (N = 2048) row segments.
// The arithmetic is the plain kernels' (same radix order, twiddle tables and
// rounding), so the results are bit-identical to schedule 0.  The wait for a
// tile is bounded: on expiry the kernel records GLSFFT_ERROR_TIMEOUT in the
// context's device status word, waits (bounded) for its copy in flight and
// returns.  Row variants of the same design measured slower than row
// schedule 2 and are not built.
#include <cuda.h>

#include "fft_config.h"
#include "fft_kernels.cuh"
#include "glsfft.h"
#include "glsfft_internal.h"
#include "sched_internal.h"
#include "tma_device.cuh"

namespace glsfft {

namespace {

constexpr unsigned kStreamTileBytes = 128u * 1024u;
constexpr long long kStreamWaitNs = 2000000000ll;  // 2 s per tile: a safety bound only

template <int N>
__host__ __device__ constexpr int stream_lines() {
    return (int)(kStreamTileBytes / (N * sizeof(float2)));
}
template <int N>
__host__ __device__ constexpr size_t stream_xchg_bytes() {
    constexpr size_t b = sizeof(float) * (size_t)col_split_floats(stream_lines<N>() * N);
    return (b + 15) & ~size_t(15);
}
template <int N>
__host__ __device__ constexpr size_t stream_smem() {
    return 128 + kStreamTileBytes + stream_xchg_bytes<N>() + 16;
}
template <int N, int E>
__host__ __device__ constexpr int stream_threads() {
    return stream_lines<N>() * (N / E);
}

// Issue the copy of tile `tile` (image tile / tpi, columns (tile % tpi) * L
// onward) into the stage, completing on `full`.  The tensor map views the
// batch as (rows * images) x cols 8-byte elements.
template <int N>
__device__ __forceinline__ void stream_issue(const CUtensorMap *tmap, const PassArgs &a, int tile,
                                             int tpi, float2 *stage, unsigned long long *full,
                                             bool inject = false) {
    constexpr int L = stream_lines<N>();
    const int y0 = (tile / tpi) * a.rows, x = (tile % tpi) * L;
    mbar_arrive_tx(full, kStreamTileBytes);
    if (inject) return;  // fault injection: the copy is never issued
#pragma unroll
    for (int b = 0; b < N / 256; b++) tensor2d_g2s(stage + b * 256 * L, tmap, x, y0 + b * 256, full);
}

// ST: ST_C2 (complex out), or, over one image, ST_LOGMAG_MINMAX (the FFT
// display epilogue of the plain column kernel: log(|X| + param) as CV_32FC1
// and the minMaxLoc keys of what is stored, reduced over all of the block's
// tiles and committed once)
template <int N, int E, int ST>
__global__ void __launch_bounds__(stream_threads<N, E>(), 1)
    fft_stream_cols(const __grid_constant__ CUtensorMap tmap, const PassArgs a, int images) {
    constexpr int L = stream_lines<N>(), T = N / E;
    static_assert(N % 256 == 0, "column tiles are read as 256-row boxes");
    static_assert(ST == ST_C2 || ST == ST_LOGMAG_MINMAX, "stream store modes");
    extern __shared__ unsigned char stream_raw[];
    // 128-byte aligned stage; offsetting the shared array itself (not a cast
    // integer) keeps the compiler's shared-window addressing
    unsigned char *base = stream_raw + ((128u - (smem_u32(stream_raw) & 127u)) & 127u);
    float2 *stage = reinterpret_cast<float2 *>(base);
    float *xch = reinterpret_cast<float *>(base + kStreamTileBytes);
    unsigned long long *full =
        reinterpret_cast<unsigned long long *>(base + kStreamTileBytes + stream_xchg_bytes<N>());

    pdl_enter();  // before the first tile copy reads the input
    const int tid = threadIdx.x;
    const int tpi = a.cols / L;  // tiles per image
    const int total = tpi * images;
    const int l = tid % L, t = tid / L;  // column within the tile, position thread

    if (tid == 0) {
        mbar_init(full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int tile = blockIdx.x;
    const bool inject = a.stall_ns > 0;
    if (tid == 0 && tile < total) stream_issue<N>(&tmap, a, tile, tpi, stage, full, inject);
    unsigned parity = 0;
    MinMaxAny run;  // ST_LOGMAG_MINMAX only
    const long long limit = inject ? a.stall_ns : kStreamWaitNs;
    for (; tile < total; tile += gridDim.x) {
        const bool ok = mbar_wait(full, parity, limit);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                if (a.err) atomicExch(a.err, (int)GLSFFT_ERROR_TIMEOUT);
                // the copy in flight, if one was issued
                if (!inject) mbar_wait(full, parity, kStreamWaitNs);
            }
            __syncthreads();
            return;
        }
        parity ^= 1u;
        float2 x[E];
#pragma unroll
        for (int m = 0; m < E; m++) x[m] = stage[(t + m * T) * L + l];
        __syncthreads();  // every thread has its values: the stage is free
        const int next = tile + gridDim.x;
        if (tid == 0 && next < total) stream_issue<N>(&tmap, a, next, tpi, stage, full);

        conj_line(x, a.flags & PF_CONJ_IN);
        LineFft<N, E, SyncBlock, 4>::run(x, t, ColSmF<L>{xch, l}, a.tw);
        finish_line(x, a.scale, a.flags & PF_CONJ_OUT);

        const int col = (tile % tpi) * L + l;
        const int ocol = (a.flags & PF_SHIFT_COLS) ? (col + (a.cols >> 1)) & (a.cols - 1) : col;
        char *out = static_cast<char *>(a.out0) + (size_t)(tile / tpi) * a.out_img_bytes;
        if constexpr (ST == ST_LOGMAG_MINMAX) {
            float *fo = reinterpret_cast<float *>(out);
#pragma unroll
            for (int m = 0; m < E; m++) {
                const int pos = t + m * T;
                const int orow = (a.flags & PF_SHIFT_ROWS) ? (pos + (N >> 1)) & (N - 1) : pos;
                const unsigned o = (unsigned)orow * (unsigned)a.cols + (unsigned)ocol;
                const float v = spec_log_mag(x[m], a.param);
                fo[o] = v;
                run.add(v, o);
            }
        } else {
            store_line<N, E, T>(reinterpret_cast<float2 *>(out) + ocol, (size_t)a.cols, x, t,
                                a.flags & PF_SHIFT_ROWS);
        }
    }
    if constexpr (ST == ST_LOGMAG_MINMAX) {
        __shared__ unsigned long long red[2 * (stream_threads<N, E>() / 32)];
        block_minmax_commit(run.kmin(), run.kmax(), red, a.key);
    }
}

template <int N, int E, int ST>
cudaError_t stream_launch(const PassArgs &a, int images, cudaStream_t s) {
    constexpr int L = stream_lines<N>();
    CUtensorMap tmap{};
    if (make_tmap_2d(&tmap, a.in0, a.cols, (long long)a.rows * images, L, 256) != GLSFFT_SUCCESS)
        return cudaErrorNotSupported;
    constexpr size_t smem = stream_smem<N>();
    auto kern = fft_stream_cols<N, E, ST>;
    cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (sms <= 0) return cudaErrorNotSupported;
    const long long total = (long long)(a.cols / L) * images;
    const int grid = (int)(total < sms ? total : sms);
    return launch_maybe_pdl(a.pdl != 0, kern, dim3(grid), dim3(stream_threads<N, E>()), smem, s,
                            tmap, a, images);
}

}  // namespace

bool stream_pass_applies(int n, bool cols, const PassArgs &a, int images, int st) {
    if (!cols || (n != 2048 && n != 4096)) return false;
    if (a.in1 || a.out1 || !a.in0 || !a.out0 || images < 1) return false;
    if (st != ST_C2 && !(st == ST_LOGMAG_MINMAX && images == 1 && a.key)) return false;
    const int L = (int)(kStreamTileBytes / (n * sizeof(float2)));
    if (a.rows != n || a.cols < L || a.cols % L) return false;
    const size_t img = (size_t)a.rows * a.cols * sizeof(float2);
    if (images > 1 && (a.in_img_bytes != img || a.out_img_bytes != img)) return false;
    const uintptr_t in = reinterpret_cast<uintptr_t>(a.in0), out = reinterpret_cast<uintptr_t>(a.out0);
    return (in % 16) == 0 && (out % (st == ST_C2 ? 16 : 4)) == 0;
}

cudaError_t launch_stream_pass(int n, bool cols, const PassArgs &a, int images, cudaStream_t s,
                               int st) {
    if (!stream_pass_applies(n, cols, a, images, st)) return cudaErrorNotSupported;
    // 16 values per thread (1024 threads); 32 per thread (512 threads)
    // measured the same on GB300
    if (st == ST_LOGMAG_MINMAX)
        return n == 2048 ? stream_launch<2048, 16, ST_LOGMAG_MINMAX>(a, images, s)
                         : stream_launch<4096, 16, ST_LOGMAG_MINMAX>(a, images, s);
    return n == 2048 ? stream_launch<2048, 16, ST_C2>(a, images, s)
                     : stream_launch<4096, 16, ST_C2>(a, images, s);
}

}  // namespace glsfft
