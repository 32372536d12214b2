// fft_stream.cu -- streamed row and column passes for 2048- and 4096-point
// lines (pass schedule kSchedStreamed).
//
// A tile of the plain column kernel for 4096-point columns (4 columns, 32
// bytes of each image row) is 128 KB, so an SM holds one tile at a time and
// loads, transforms and stores it in turn: HBM idles while the SM computes.
// Here one persistent 1024-thread block per SM walks the tiles of the pass
// (image-major, then tile) and keeps the NEXT tile's copy in flight while it
// transforms the current one:
//   * the tile (L lines, L * N * 8 = 128 KB) lands in a shared-memory stage
//     through the Tensor Memory Accelerator -- one cp.async.bulk per row for
//     a rows tile, N/256 2-D tensor boxes of L x 256 for a columns tile --
//     completing on an mbarrier;
//   * every thread copies its 16 values of one line to registers, the block
//     syncs, and thread 0 at once issues the next tile's copy into the stage;
//   * the Stockham passes exchange through a separate float buffer, real and
//     imaginary parts in turn (half the shared memory of a complex exchange,
//     so stage + exchange fit one SM: 128 KB + 66-70 KB);
//   * results are stored from registers in the image layout (whole 32- or
//     64-byte row segments for a columns tile, whole rows for a rows tile).
// The arithmetic is the plain kernels' (same radix order, twiddle tables and
// rounding), so the results are bit-identical to schedule 0.  The wait for a
// tile is bounded: on expiry the kernel records GLSFFT_ERROR_TIMEOUT in the
// context's device status word, waits (bounded) for its copy in flight and
// returns.
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
template <int N, bool COLS>
__host__ __device__ constexpr size_t stream_xchg_bytes() {
    constexpr int L = stream_lines<N>();
    constexpr size_t b = sizeof(float) * (size_t)(COLS ? col_split_floats(L * N) : L * row_split_floats(N));
    return (b + 15) & ~size_t(15);
}
template <int N, bool COLS>
__host__ __device__ constexpr size_t stream_smem() {
    return 128 + kStreamTileBytes + stream_xchg_bytes<N, COLS>() + 16;
}

// Issue the copy of tile `tile` (image tile / tpi, tile tile % tpi of it)
// into the stage, completing on `full`.
template <int N, bool COLS>
__device__ __forceinline__ void stream_issue(const CUtensorMap *tmap, const PassArgs &a, int tile,
                                             int tpi, float2 *stage, unsigned long long *full) {
    constexpr int L = stream_lines<N>();
    const int img = tile / tpi, j = tile % tpi;
    mbar_arrive_tx(full, kStreamTileBytes);
    if constexpr (COLS) {
        // columns j*L .. j*L+L-1 of image img: the tensor map views the batch
        // as (rows * images) x cols 8-byte elements
        const int y0 = img * a.rows;
#pragma unroll
        for (int b = 0; b < N / 256; b++)
            tensor2d_g2s(stage + b * 256 * L, tmap, j * L, y0 + b * 256, full);
    } else {
        const char *src = static_cast<const char *>(a.in0) + (size_t)img * a.in_img_bytes +
                          (size_t)j * L * N * sizeof(float2);
#pragma unroll
        for (int l = 0; l < L; l++)
            bulk_g2s(stage + l * N, src + (size_t)l * N * sizeof(float2), N * sizeof(float2), full);
    }
}

template <int N, int E>
__host__ __device__ constexpr int stream_threads() {
    return stream_lines<N>() * (N / E);
}

// ST: ST_C2 (complex out), or, for a column pass over one image,
// ST_LOGMAG_MINMAX (the FFT display epilogue of the plain column kernel:
// log(|X| + param) as CV_32FC1 and the minMaxLoc keys of what is stored,
// reduced over all of the block's tiles and committed once)
template <int N, int E, bool COLS, int ST>
__global__ void __launch_bounds__(stream_threads<N, E>(), 1)
    fft_stream_kernel(const __grid_constant__ CUtensorMap tmap, const PassArgs a, int images) {
    constexpr int L = stream_lines<N>(), T = N / E;
    static_assert(ST == ST_C2 || (COLS && ST == ST_LOGMAG_MINMAX), "stream store modes");
    static_assert(N % 256 == 0, "column tiles are read as 256-row boxes");
    extern __shared__ unsigned char stream_raw[];
    // 128-byte aligned stage; offsetting the shared array itself (not a cast
    // integer) keeps the compiler's shared-window addressing
    unsigned char *base = stream_raw + ((128u - (smem_u32(stream_raw) & 127u)) & 127u);
    float2 *stage = reinterpret_cast<float2 *>(base);
    float *xch = reinterpret_cast<float *>(base + kStreamTileBytes);
    unsigned long long *full =
        reinterpret_cast<unsigned long long *>(base + kStreamTileBytes + stream_xchg_bytes<N, COLS>());

    const int tid = threadIdx.x;
    const int tpi = (COLS ? a.cols : a.rows) / L;  // tiles per image
    const int total = tpi * images;
    // line within the tile (column offset for columns) and position thread
    const int l = COLS ? tid % L : tid / T;
    const int t = COLS ? tid / L : tid % T;

    if (tid == 0) {
        mbar_init(full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int tile = blockIdx.x;
    if (tid == 0 && tile < total) stream_issue<N, COLS>(&tmap, a, tile, tpi, stage, full);
    unsigned parity = 0;
    MinMaxAny run;  // ST_LOGMAG_MINMAX only
    for (; tile < total; tile += gridDim.x) {
        const bool ok = mbar_wait(full, parity, kStreamWaitNs);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                if (a.err) atomicExch(a.err, (int)GLSFFT_ERROR_TIMEOUT);
                mbar_wait(full, parity, kStreamWaitNs);  // the copy in flight
            }
            __syncthreads();
            return;
        }
        parity ^= 1u;
        float2 x[E];
#pragma unroll
        for (int m = 0; m < E; m++)
            x[m] = COLS ? stage[(t + m * T) * L + l] : stage[l * N + t + m * T];
        __syncthreads();  // every thread has its values: the stage is free
        const int next = tile + gridDim.x;
        if (tid == 0 && next < total) stream_issue<N, COLS>(&tmap, a, next, tpi, stage, full);

        conj_line(x, a.flags & PF_CONJ_IN);
        using F = LineFft<N, E, SyncBlock, 4>;
        if constexpr (COLS)
            F::run(x, t, ColSmF<L>{xch, l}, a.tw);
        else
            F::run(x, t, RowSmF{xch + l * row_split_floats(N)}, a.tw);
        finish_line(x, a.scale, a.flags & PF_CONJ_OUT);

        const int img = tile / tpi, j = tile % tpi;
        float2 *out = reinterpret_cast<float2 *>(static_cast<char *>(a.out0) +
                                                 (size_t)img * a.out_img_bytes);
        if constexpr (ST == ST_LOGMAG_MINMAX) {
            const int col = j * L + l;
            const int ocol = (a.flags & PF_SHIFT_COLS) ? (col + (a.cols >> 1)) & (a.cols - 1) : col;
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
        } else if constexpr (COLS) {
            const int col = j * L + l;
            const int ocol = (a.flags & PF_SHIFT_COLS) ? (col + (a.cols >> 1)) & (a.cols - 1) : col;
            store_line<N, E, T>(out + ocol, (size_t)a.cols, x, t, a.flags & PF_SHIFT_ROWS);
        } else {
            const int row = j * L + l;
            const int orow = (a.flags & PF_SHIFT_ROWS) ? (row + (a.rows >> 1)) & (a.rows - 1) : row;
            store_line<N, E, T>(out + (size_t)orow * N, 1, x, t, a.flags & PF_SHIFT_COLS);
        }
    }
    if constexpr (ST == ST_LOGMAG_MINMAX) {
        __shared__ unsigned long long red[2 * (stream_threads<N, E>() / 32)];
        block_minmax_commit(run.kmin(), run.kmax(), red, a.key);
    }
}

int sm_count(int device) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return v;
}

template <int N, int E, bool COLS, int ST = ST_C2>
cudaError_t stream_launch(const PassArgs &a, int images, cudaStream_t s) {
    constexpr int L = stream_lines<N>();
    CUtensorMap tmap{};
    if constexpr (COLS) {
        if (make_tmap_2d(&tmap, a.in0, a.cols, (long long)a.rows * images, L, 256) != GLSFFT_SUCCESS)
            return cudaErrorNotSupported;
    }
    constexpr size_t smem = stream_smem<N, COLS>();
    auto kern = fft_stream_kernel<N, E, COLS, ST>;
    cudaError_t e = smem_opt_in(reinterpret_cast<const void *>(kern), smem);
    if (e != cudaSuccess) return e;
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int sms = sm_count(dev);
    if (sms <= 0) return cudaErrorNotSupported;
    const long long total = (long long)((COLS ? a.cols : a.rows) / L) * images;
    const int grid = (int)(total < sms ? total : sms);
    kern<<<grid, stream_threads<N, E>(), smem, s>>>(tmap, a, images);
    return cudaGetLastError();
}

}  // namespace

bool stream_pass_applies(int n, bool cols, const PassArgs &a, int images, int st) {
    if (n != 2048 && n != 4096) return false;
    if (a.in1 || a.out1 || !a.in0 || !a.out0 || images < 1) return false;
    if (st != ST_C2 && !(st == ST_LOGMAG_MINMAX && cols && images == 1 && a.key)) return false;
    const int L = (int)(kStreamTileBytes / (n * sizeof(float2)));
    const int other = cols ? a.cols : a.rows;  // lines in the pass
    if ((cols ? a.rows : a.cols) != n || other < L || other % L) return false;
    const size_t img = (size_t)a.rows * a.cols * sizeof(float2);
    if (images > 1 && (a.in_img_bytes != img || a.out_img_bytes != img)) return false;
    const uintptr_t in = reinterpret_cast<uintptr_t>(a.in0), out = reinterpret_cast<uintptr_t>(a.out0);
    return (in % 16) == 0 && (out % (st == ST_C2 ? 16 : 4)) == 0;
}

cudaError_t launch_stream_pass(int n, bool cols, const PassArgs &a, int images, cudaStream_t s,
                               int st) {
    if (!stream_pass_applies(n, cols, a, images, st)) return cudaErrorNotSupported;
    if (st == ST_LOGMAG_MINMAX)
        return n == 2048 ? stream_launch<2048, 16, true, ST_LOGMAG_MINMAX>(a, images, s)
                         : stream_launch<4096, 16, true, ST_LOGMAG_MINMAX>(a, images, s);
    // 16 values per thread (1024 threads); 32 per thread (512 threads)
    // measured the same on GB300
    if (n == 2048) return cols ? stream_launch<2048, 16, true>(a, images, s) : stream_launch<2048, 16, false>(a, images, s);
    return cols ? stream_launch<4096, 16, true>(a, images, s) : stream_launch<4096, 16, false>(a, images, s);
}

}  // namespace glsfft
