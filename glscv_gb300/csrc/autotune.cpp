// autotune.cpp -- the plain path's autotuner.  For one image size it times
// every available schedule of the complex row pass and of the column pass
// (radix bound, elements per thread, lines or columns per block:
// fft_config.h) on scratch buffers, keeps the fastest of each in the
// context for that size, and records the choice in an optional plan cache
// file (plan_cache.h) from which a later process takes it without timing.
// The reference has no counterpart: its GLSL path runs one fixed radix-4
// schedule (glsCV/glsFft.cpp:494-671).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "fft_config.h"
#include "glsfft.h"
#include "glsfft_internal.h"
#include "sched_internal.h"

using namespace glsfft;

namespace {

// a non-default schedule must beat schedule 0 by this fraction to be kept,
// so timing noise does not flip the choice between equivalent schedules
constexpr double kKeepMargin = 0.01;

std::string num(long long v) { return std::to_string(v); }

std::string fmt_ms(double v) {
    char b[32];
    std::snprintf(b, sizeof b, "%.6g", v);
    return b;
}

}  // namespace

plan_cache::Pairs glsfft::device_fields(int device) {
    cudaDeviceProp p{};
    int drv = 0, rt = 0;
    cudaGetDeviceProperties(&p, device);
    cudaDriverGetVersion(&drv);
    cudaRuntimeGetVersion(&rt);
    cudaGetLastError();
    return {{"device", plan_cache::quote(p.name)},
            {"sms", num(p.multiProcessorCount)},
            {"cc", plan_cache::quote(num(p.major) + "." + num(p.minor))},
            {"driver", num(drv)},
            {"runtime", num(rt)},
            {"lib", num(glsfft_version())}};
}

int glsfft::time_median_ms(const std::function<int()> &fn, int warm, int reps, cudaStream_t s,
                           double *ms) {
    for (int i = 0; i < warm; i++) {
        const int st = fn();
        if (st) return st;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int st = cuda_status(e);
    std::vector<double> t;
    for (int i = 0; i < reps && !st; i++) {
        e = cudaEventRecord(e0, s);
        if (e == cudaSuccess) {
            st = fn();
            if (!st) e = cudaEventRecord(e1, s);
        }
        if (!st && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float f = 0.f;
        if (!st && e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
        if (!st) st = cuda_status(e);
        t.push_back(f);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) return st;
    std::sort(t.begin(), t.end());
    *ms = t.empty() ? 0.0 : t[t.size() / 2];
    return GLSFFT_SUCCESS;
}

extern "C" {

int glsfft_schedule_available(int length, int schedule, int along_cols) {
    if (length < 1 || length > kMaxLen || (length & (length - 1))) return 0;
    if (schedule == 0) return 1;
    if (schedule < 0 || schedule >= kPassSchedules || length < kSchedMinLen) return 0;
    // the constexpr table evaluated at run time
    return sched_available(length, schedule, along_cols != 0) ? 1 : 0;
}

int glsfft_set_fft_schedule(glsfft_context ctx, int rows, int cols, int row_schedule,
                            int col_schedule) {
    if (!ctx) return GLSFFT_ERROR_INVALID_VALUE;
    const int st = check_dims(rows, cols);
    if (st) return st;
    if (!glsfft_schedule_available(cols, row_schedule, 0) ||
        !glsfft_schedule_available(rows, col_schedule, 1))
        return GLSFFT_ERROR_INVALID_VALUE;
    const FftSchedule d = default_schedule(rows, cols);
    if (row_schedule == d.row && col_schedule == d.col)
        ctx->sched.erase(sched_key(rows, cols));
    else
        ctx->sched[sched_key(rows, cols)] = FftSchedule{row_schedule, col_schedule};
    return GLSFFT_SUCCESS;
}

int glsfft_get_fft_schedule(glsfft_context ctx, int rows, int cols, int *row_schedule,
                            int *col_schedule) {
    if (!ctx || !row_schedule || !col_schedule) return GLSFFT_ERROR_INVALID_VALUE;
    const int st = check_dims(rows, cols);
    if (st) return st;
    const FftSchedule sc = schedule_for(ctx->sched, rows, cols);
    *row_schedule = sc.row;
    *col_schedule = sc.col;
    return GLSFFT_SUCCESS;
}

int glsfft_autotune_fft2d(glsfft_context ctx, int rows, int cols, int count,
                          const char *cache_path, void *stream, int *result, double *ms) {
    if (!ctx || count < 1 || count > kMaxBatch) return GLSFFT_ERROR_INVALID_VALUE;
    int st = check_dims(rows, cols);
    if (st) return st;
    DeviceGuard g(ctx->device);
    if (!g.ok()) return GLSFFT_ERROR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    int res[3] = {0, 0, 0};
    double t[2] = {0.0, 0.0};

    plan_cache::Pairs key = device_fields(ctx->device);
    key.push_back({"kind", plan_cache::quote("fft2d")});
    key.push_back({"rows", num(rows)});
    key.push_back({"cols", num(cols)});
    key.push_back({"count", num(count)});
    plan_cache::Fields hit;
    if (plan_cache::lookup(cache_path, plan_cache::as_fields(key), hit)) {
        const int r = std::atoi(hit["row_schedule"].c_str());
        const int c = std::atoi(hit["col_schedule"].c_str());
        if (glsfft_schedule_available(cols, r, 0) && glsfft_schedule_available(rows, c, 1)) {
            st = glsfft_set_fft_schedule(ctx, rows, cols, r, c);
            if (st) return st;
            res[0] = r;
            res[1] = c;
            res[2] = 1;
            t[0] = std::atof(hit["ms"].c_str());
            t[1] = std::atof(hit["ms_default"].c_str());
            if (result) std::copy(res, res + 3, result);
            if (ms) std::copy(t, t + 2, ms);
            return GLSFFT_SUCCESS;
        }
    }

    const size_t bytes = (size_t)count * rows * cols * sizeof(float2);
    if (ctx->budget && 2 * bytes > ctx->budget) return GLSFFT_ERROR_BUDGET;
    void *src = nullptr, *dst = nullptr;
    cudaError_t e = cudaMalloc(&src, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dst, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(src, 0x3f, bytes, s);  // finite values
    st = cuda_status(e);

    PassArgs a{};
    a.in0 = src;
    a.out0 = dst;
    a.rows = rows;
    a.cols = cols;
    a.scale = 1.0f;
    a.tw = ctx->d_tw;
    a.in_img_bytes = a.out_img_bytes = (size_t)rows * cols * sizeof(float2);
    // each pass: its default schedule first, then the others in order; the
    // fastest is kept unless the default is within kKeepMargin of it
    const FftSchedule dflt = default_schedule(rows, cols);
    for (int along_cols = 0; along_cols < 2 && !st; along_cols++) {
        const int n = along_cols ? rows : cols;
        const int first = along_cols ? dflt.col : dflt.row;
        double best = 0.0, base = 0.0;
        int best_id = first;
        for (int k = -1; k < kPassSchedules && !st; k++) {
            const int id = k < 0 ? first : k;
            if ((k >= 0 && id == first) || !glsfft_schedule_available(n, id, along_cols)) continue;
            double m = 0.0;
            st = time_median_ms(
                [&]() {
                    return cuda_status(along_cols ? launch_cols_sched(n, id, a, count, s)
                                                  : launch_rows_sched(n, id, a, count, s));
                },
                2, 7, s, &m);
            if (st) break;
            if (k < 0) {
                base = best = m;
            } else if (m < best && m < base * (1.0 - kKeepMargin)) {
                best = m;
                best_id = id;
            }
        }
        res[along_cols] = best_id;
        t[0] += best;
        t[1] += base;
    }
    if (src || dst) {
        cudaStreamSynchronize(s);
        if (src) cudaFree(src);
        if (dst) cudaFree(dst);
        cudaGetLastError();
    }
    if (st) return st;
    st = glsfft_set_fft_schedule(ctx, rows, cols, res[0], res[1]);
    if (st) return st;
    if (cache_path && *cache_path) {
        key.push_back({"row_schedule", num(res[0])});
        key.push_back({"col_schedule", num(res[1])});
        key.push_back({"ms", fmt_ms(t[0])});
        key.push_back({"ms_default", fmt_ms(t[1])});
        if (!plan_cache::append(cache_path, key)) st = GLSFFT_ERROR_IO;
    }
    if (result) std::copy(res, res + 3, result);
    if (ms) std::copy(t, t + 2, ms);
    return st;
}

}  // extern "C"
