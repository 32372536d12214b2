// noalloc.cu -- glsfft_phase_correlate_noalloc: phaseCorrelate for callers
// that may not allocate device memory.  Its scratch and twiddle table are
// file-scope static device arrays; host code reaches them only through the
// device addresses cudaGetSymbolAddress returns (the array names are host
// stand-ins in host code, not device addresses).
#include <cstdint>
#include <mutex>

#include "capi_internal.h"
#include "glsfft_internal.h"

namespace {

constexpr size_t kMaxPixels = GLSFFT_NOALLOC_MAX_PIXELS;
// F1 | F2 (complex) | surface (float) | argmax word, laid out as poc_launch
// expects for any rows*cols <= kMaxPixels.
constexpr size_t kKeyOffset = (20 * kMaxPixels + 255) / 256 * 256;
constexpr size_t kScratchBytes = kKeyOffset + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];
static __device__ __align__(256) float2 g_noalloc_twiddles[glsfft::kTwEntries];

struct DeviceSetup {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    float2 *twiddles = nullptr;        // device address of g_noalloc_twiddles
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];
float2 g_host_twiddles[glsfft::kTwEntries];  // staging for the one upload

// Once per device, with that device current.
int setup_current_device(DeviceSetup **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return glsfft::cuda_status(e);
    if (dev < 0 || dev >= kMaxDevices) return GLSFFT_ERROR_INVALID_VALUE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup &s = g_setup[dev];
    if (!s.ready) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return glsfft::cuda_status(e);
        s.scratch = static_cast<unsigned char *>(p);
        e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
        if (e != cudaSuccess) return glsfft::cuda_status(e);
        s.twiddles = static_cast<float2 *>(p);
        glsfft::make_twiddle_host(g_host_twiddles);
        e = cudaMemcpyToSymbol(g_noalloc_twiddles, g_host_twiddles, sizeof(g_host_twiddles));
        if (e != cudaSuccess) return glsfft::cuda_status(e);
        s.ready = true;
    }
    *out = &s;
    return GLSFFT_SUCCESS;
}

inline bool pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

}  // namespace

extern "C" int glsfft_phase_correlate_noalloc(const float *src1, const float *src2,
                                              const float *window, int rows, int cols, int box,
                                              double *d_result, void *stream) {
    if (!src1 || !src2 || !d_result || box < 1) return GLSFFT_ERROR_INVALID_VALUE;
    if (rows < 1 || cols < 1 || rows > glsfft::kMaxLen || cols > glsfft::kMaxLen)
        return GLSFFT_ERROR_SIZE;
    if (!pow2(rows) || !pow2(cols)) return GLSFFT_ERROR_NOT_POW2;
    const size_t n = (size_t)rows * cols;
    if (n > kMaxPixels) return GLSFFT_ERROR_NOALLOC_LIMIT;
    if ((reinterpret_cast<uintptr_t>(src1) & 3) || (reinterpret_cast<uintptr_t>(src2) & 3) ||
        (window && (reinterpret_cast<uintptr_t>(window) & 3)) ||
        (reinterpret_cast<uintptr_t>(d_result) & 7))
        return GLSFFT_ERROR_MISALIGNED;
    DeviceSetup *s = nullptr;
    int st = setup_current_device(&s);
    if (st) return st;
    float2 *f1 = reinterpret_cast<float2 *>(s->scratch);
    float2 *f2 = f1 + n;
    float *surface = reinterpret_cast<float *>(f2 + n);
    auto *key = reinterpret_cast<unsigned long long *>(s->scratch + kKeyOffset);
    // poc_launch clears the argmax word before the kernels run
    return glsfft::poc_launch(s->twiddles, src1, src2, window, rows, cols, box, f1, f2, surface,
                              key, d_result, (cudaStream_t)stream);
}
