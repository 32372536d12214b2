// noalloc.cu -- glsfft_phase_correlate_noalloc: phaseCorrelate for callers
// that may not allocate device memory.  Its scratch and twiddle table are
// file-scope static device arrays; host code reaches them only through the
// device addresses cudaGetSymbolAddress returns (the array names are host
// stand-ins in host code, not device addresses).
#include <cuda.h>
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
    unsigned long long context_id = 0;  // the CUDA context the addresses belong to
    unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch
    float2 *twiddles = nullptr;         // device address of g_noalloc_twiddles
};

// The set-up is cached per CUDA context, not per device ordinal: after a
// cudaDeviceReset, or on another driver context of the same device, the
// module's static arrays are fresh (zeroed, possibly at other addresses), so
// a new context id redoes the address lookup and the twiddle upload.
constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxContexts];
int g_setup_next = 0;  // round-robin replacement once every entry is used
float2 g_host_twiddles[glsfft::kTwEntries];  // staging for the upload

using CtxGetCurrent = CUresult (*)(CUcontext *);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long *);

void *driver_entry(const char *name, int version) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        return nullptr;
    return p;
}

// The id of the calling thread's current CUDA context (0 on failure).
unsigned long long current_context_id() {
    static std::once_flag once;
    static CtxGetCurrent get_current = nullptr;
    static CtxGetId get_id = nullptr;
    std::call_once(once, [] {
        get_current = reinterpret_cast<CtxGetCurrent>(driver_entry("cuCtxGetCurrent", 4000));
        get_id = reinterpret_cast<CtxGetId>(driver_entry("cuCtxGetId", 12000));
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Once per CUDA context, with that context current (the current device's
// primary context for runtime-API callers).
int setup_current_context(DeviceSetup *out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return glsfft::cuda_status(e);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = current_context_id();
    if (id != 0)
        for (const DeviceSetup &s : g_setup)
            if (s.context_id == id) {
                *out = s;
                return GLSFFT_SUCCESS;
            }
    // the lookup also makes the runtime's primary context current when this
    // thread has none yet
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return glsfft::cuda_status(e);
    DeviceSetup s;
    s.scratch = static_cast<unsigned char *>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
    if (e != cudaSuccess) return glsfft::cuda_status(e);
    s.twiddles = static_cast<float2 *>(p);
    glsfft::make_twiddle_host(g_host_twiddles);
    e = cudaMemcpyToSymbol(g_noalloc_twiddles, g_host_twiddles, sizeof(g_host_twiddles));
    if (e != cudaSuccess) return glsfft::cuda_status(e);
    if (id == 0) id = current_context_id();
    if (id == 0) return GLSFFT_ERROR_CUDA;
    s.context_id = id;
    g_setup[g_setup_next] = s;
    g_setup_next = (g_setup_next + 1) % kMaxContexts;
    *out = s;
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
    DeviceSetup setup;
    int st = setup_current_context(&setup);
    if (st) return st;
    const DeviceSetup *s = &setup;
    float2 *f1 = reinterpret_cast<float2 *>(s->scratch);
    float2 *f2 = f1 + n;
    float *surface = reinterpret_cast<float *>(f2 + n);
    auto *key = reinterpret_cast<unsigned long long *>(s->scratch + kKeyOffset);
    // poc_launch clears the argmax word before the kernels run
    return glsfft::poc_launch(s->twiddles, src1, src2, window, rows, cols, box, f1, f2, surface,
                              key, d_result, (cudaStream_t)stream);
}
