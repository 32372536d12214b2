// spectrum_device.cuh -- element formulas of the spectrum operations and the
// minMaxLoc keys, shared by the standalone kernels (spectrum.cu) and the
// fused column-pass epilogue of the FFT display pipeline.
//
// Formulas follow the reference shaders (glsCV/glsBasicOperation.cpp:153-212
// binary ops 6-8, :92-141 scalar ops 9 and 13) with every product, sum and
// quotient rounded separately (no contraction), as a C restatement compiled
// with -ffp-contract=off computes them.
#pragma once
#include <cuda_runtime.h>

#include <cstring>

namespace glsfft {

// mulSpectrums: a*b, or a*conj(b) (OPCODE_MUL_SPCETRUM / _CONJ)
template <bool CONJ>
__device__ __forceinline__ float2 spec_mul(float2 a, float2 b) {
    if constexpr (CONJ)
        return make_float2(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                           __fadd_rn(__fmul_rn(-a.x, b.y), __fmul_rn(a.y, b.x)));
    else
        return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                           __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
// mulSpectrumsPhaseOnly: t = a*conj(b), t / |t|, no epsilon (0/0 is NaN)
__device__ __forceinline__ float2 spec_poc(float2 a, float2 b) {
    const float2 t = spec_mul<true>(a, b);
    const float mag = sqrtf(__fadd_rn(__fmul_rn(t.x, t.x), __fmul_rn(t.y, t.y)));
    return make_float2(__fdiv_rn(t.x, mag), __fdiv_rn(t.y, mag));
}
// magSpectrums: sqrt(re^2 + im^2)
__device__ __forceinline__ float spec_mag(float2 a) {
    return sqrtf(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
}
// logMagSpectrums: log(|sqrt(re^2 + im^2) + offset|)
__device__ __forceinline__ float spec_log_mag(float2 a, float offset) {
    return logf(fabsf(__fadd_rn(spec_mag(a), offset)));
}

// ------------------------------------------------------------ minMaxLoc keys
// gls::minMaxLoc (glsCV/glsMinMaxLoc.cpp:65-119) scans with strict compares
// from the shader's FLT_MAX literal, so the result is the first occurrence in
// row-major order among the elements below (above) the literal; NaN never
// compares.  A 64-bit key per element -- order-preserving value bits, then
// the complement of the row-major index -- makes that an atomicMax: the
// extreme value wins, ties go to the smallest index.  Key 0 means "none".
constexpr float kMinMaxLiteral = 3.402823e+38f;

__device__ __forceinline__ unsigned ord_bits(float v) {
    const unsigned b = __float_as_uint(__fadd_rn(v, 0.0f));  // -0 compares equal to +0
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long max_key(float v, unsigned idx) {
    if (!(v > -kMinMaxLiteral)) return 0ull;
    return ((unsigned long long)ord_bits(v) << 32) | (unsigned long long)(0xFFFFFFFFu - idx);
}
__device__ __forceinline__ unsigned long long min_key(float v, unsigned idx) {
    if (!(v < kMinMaxLiteral)) return 0ull;
    return ((unsigned long long)(~ord_bits(v)) << 32) | (unsigned long long)(0xFFFFFFFFu - idx);
}
__host__ __device__ inline float ord_value(unsigned o) {
    const unsigned b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
}
// value and index of a key (none: the literal at index 0)
__host__ __device__ inline float max_key_value(unsigned long long k) {
    return k ? ord_value((unsigned)(k >> 32)) : -kMinMaxLiteral;
}
__host__ __device__ inline float min_key_value(unsigned long long k) {
    return k ? ord_value(~(unsigned)(k >> 32)) : kMinMaxLiteral;
}
__host__ __device__ inline unsigned key_idx(unsigned long long k) {
    return k ? 0xFFFFFFFFu - (unsigned)(k & 0xFFFFFFFFull) : 0u;
}

// Running min / max of one thread over indices visited in any order: strict
// compares, equal values resolved to the smaller index; keys are formed once
// at the end (values at the literal, which the tie rule may have taken, give
// no key).
struct MinMaxAny {
    float vmin = kMinMaxLiteral, vmax = -kMinMaxLiteral;
    unsigned imin = 0xFFFFFFFFu, imax = 0xFFFFFFFFu;
    __device__ __forceinline__ void add(float v, unsigned i) {
        if (v < vmin || (v == vmin && i < imin)) {
            vmin = v;
            imin = i;
        }
        if (v > vmax || (v == vmax && i < imax)) {
            vmax = v;
            imax = i;
        }
    }
    __device__ __forceinline__ unsigned long long kmin() const { return min_key(vmin, imin); }
    __device__ __forceinline__ unsigned long long kmax() const { return max_key(vmax, imax); }
};

// Block-wide max of both keys; thread 0 issues the atomics.  `red` holds
// 2 * (blockDim.x / 32) entries of shared memory.
__device__ __forceinline__ void block_minmax_commit(unsigned long long kmin,
                                                    unsigned long long kmax,
                                                    unsigned long long *red,
                                                    unsigned long long *dst2) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmin, off);
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, kmax, off);
        kmin = a > kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[warp] = kmin;
        red[warps + warp] = kmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bmin = 0, bmax = 0;
        for (int w = 0; w < warps; w++) {
            bmin = red[w] > bmin ? red[w] : bmin;
            bmax = red[warps + w] > bmax ? red[warps + w] : bmax;
        }
        if (bmin) atomicMax(dst2, bmin);
        if (bmax) atomicMax(dst2 + 1, bmax);
    }
}

}  // namespace glsfft
