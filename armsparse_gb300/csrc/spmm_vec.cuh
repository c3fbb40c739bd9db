// Vector access to rows of B for the SpMM kernels (sm_103a): fp32 or bf16 storage, 2..16-byte
// loads, fp32 arithmetic. Included by the kernel files only.
#pragma once

#include "common.cuh"

namespace as {
namespace {

// Vector loads of B: Raw is the register form a load lands in (bf16 stays packed until the
// FMA that consumes it, so a deep unroll keeps more bytes in flight per register).
template <typename T, int VB>
struct Vec;
template <>
struct Vec<float, 16> {
    static constexpr int E = 4;
    using Raw = float4;
    __device__ static Raw raw(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
    __device__ static float at(const Raw &r, int i) {
        return i == 0 ? r.x : i == 1 ? r.y : i == 2 ? r.z : r.w;
    }
    __device__ static void load(const float *p, float *o) {
        const Raw r = raw(p);
        o[0] = r.x; o[1] = r.y; o[2] = r.z; o[3] = r.w;
    }
};
template <>
struct Vec<float, 8> {
    static constexpr int E = 2;
    using Raw = float2;
    __device__ static Raw raw(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }
    __device__ static float at(const Raw &r, int i) { return i == 0 ? r.x : r.y; }
    __device__ static void load(const float *p, float *o) {
        const Raw r = raw(p);
        o[0] = r.x; o[1] = r.y;
    }
};
template <>
struct Vec<float, 4> {
    static constexpr int E = 1;
    using Raw = float;
    __device__ static Raw raw(const float *p) { return __ldg(p); }
    __device__ static float at(const Raw &r, int) { return r; }
    __device__ static void load(const float *p, float *o) { o[0] = __ldg(p); }
};
__device__ __forceinline__ float bf16_lo(unsigned w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(unsigned w) { return __uint_as_float(w & 0xffff0000u); }

// acc_lo += lo(w) * v, acc_hi += hi(w) * v with bf16 w halves and bf16 v, fp32 accumulators:
// the mixed-precision FMA of sm_100+ (the product of two bf16 values is exact in fp32, so each
// step equals fmaf(float(b), float(v), acc) -- the same chain -- without separate unpacking).
__device__ __forceinline__ void fma_bf16x2(unsigned w, unsigned short v, float &acc_lo,
                                           float &acc_hi) {
    asm("{\n .reg .b16 l, h;\n mov.b32 {l, h}, %2;\n fma.rn.f32.bf16 %0, l, %3, %0;\n"
        " fma.rn.f32.bf16 %1, h, %3, %1;\n}\n"
        : "+f"(acc_lo), "+f"(acc_hi) : "r"(w), "h"(v));
}
// acc[i] = fmaf(b[i], v, acc[i]) for the E elements of one vector, two at a time with the
// packed fp32x2 FMA of sm_100+ (two independent round-to-nearest FMAs: the same bits as two
// fmaf calls, half the issued instructions).
template <int E>
__device__ __forceinline__ void fma_vec_f32(const float *b, float v, float *acc) {
#pragma unroll
    for (int i = 0; i + 1 < E; i += 2) {
        unsigned long long a2, b2, v2;
        asm("mov.b64 %0, {%1, %2};" : "=l"(a2) : "f"(acc[i]), "f"(acc[i + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(b2) : "f"(b[i]), "f"(b[i + 1]));
        asm("mov.b64 %0, {%1, %1};" : "=l"(v2) : "f"(v));
        asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(a2) : "l"(b2), "l"(v2));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(acc[i]), "=f"(acc[i + 1]) : "l"(a2));
    }
    if constexpr (E % 2) acc[E - 1] = fmaf(b[E - 1], v, acc[E - 1]);
}

__device__ __forceinline__ void fma_bf16x1(unsigned short b, unsigned short v, float &acc) {
    asm("fma.rn.f32.bf16 %0, %1, %2, %0;\n" : "+f"(acc) : "h"(b), "h"(v));
}
// d = fma(lo(b), lo(f), d); d = fma(hi(b), hi(f), d): one step of a dot product over two bf16
// pairs with the mixed-precision FMA (each step equals fmaf on the widened values).
__device__ __forceinline__ void dot_bf16x2(unsigned b, unsigned f, float &d) {
    asm("{\n .reg .b16 bl, bh, fl, fh;\n mov.b32 {bl, bh}, %1;\n mov.b32 {fl, fh}, %2;\n"
        " fma.rn.f32.bf16 %0, bl, fl, %0;\n fma.rn.f32.bf16 %0, bh, fh, %0;\n}\n"
        : "+f"(d) : "r"(b), "r"(f));
}
template <>
struct Vec<uint16_t, 16> {
    static constexpr int E = 8;
    using Raw = uint4;
    __device__ static Raw raw(const uint16_t *p) { return __ldg(reinterpret_cast<const uint4 *>(p)); }
    __device__ static float at(const Raw &r, int i) {
        const unsigned w = (i >> 1) == 0 ? r.x : (i >> 1) == 1 ? r.y : (i >> 1) == 2 ? r.z : r.w;
        return (i & 1) ? bf16_hi(w) : bf16_lo(w);
    }
    __device__ static void load(const uint16_t *p, float *o) {
        const Raw r = raw(p);
#pragma unroll
        for (int i = 0; i < 8; ++i) o[i] = at(r, i);
    }
    __device__ static void fma(const Raw &r, unsigned short v, float *acc) {
        fma_bf16x2(r.x, v, acc[0], acc[1]);
        fma_bf16x2(r.y, v, acc[2], acc[3]);
        fma_bf16x2(r.z, v, acc[4], acc[5]);
        fma_bf16x2(r.w, v, acc[6], acc[7]);
    }
    // d = fma chain over the elements of b and f in order
    __device__ static void dot(const Raw &b, const Raw &f, float &d) {
        dot_bf16x2(b.x, f.x, d);
        dot_bf16x2(b.y, f.y, d);
        dot_bf16x2(b.z, f.z, d);
        dot_bf16x2(b.w, f.w, d);
    }
};
template <>
struct Vec<uint16_t, 8> {
    static constexpr int E = 4;
    using Raw = uint2;
    __device__ static Raw raw(const uint16_t *p) { return __ldg(reinterpret_cast<const uint2 *>(p)); }
    __device__ static float at(const Raw &r, int i) {
        const unsigned w = (i >> 1) == 0 ? r.x : r.y;
        return (i & 1) ? bf16_hi(w) : bf16_lo(w);
    }
    __device__ static void load(const uint16_t *p, float *o) {
        const Raw r = raw(p);
#pragma unroll
        for (int i = 0; i < 4; ++i) o[i] = at(r, i);
    }
    __device__ static void fma(const Raw &r, unsigned short v, float *acc) {
        fma_bf16x2(r.x, v, acc[0], acc[1]);
        fma_bf16x2(r.y, v, acc[2], acc[3]);
    }
    __device__ static void dot(const Raw &b, const Raw &f, float &d) {
        dot_bf16x2(b.x, f.x, d);
        dot_bf16x2(b.y, f.y, d);
    }
};
template <>
struct Vec<uint16_t, 4> {
    static constexpr int E = 2;
    using Raw = unsigned;
    __device__ static Raw raw(const uint16_t *p) { return __ldg(reinterpret_cast<const unsigned *>(p)); }
    __device__ static float at(const Raw &r, int i) { return (i & 1) ? bf16_hi(r) : bf16_lo(r); }
    __device__ static void load(const uint16_t *p, float *o) {
        const Raw r = raw(p);
        o[0] = bf16_lo(r); o[1] = bf16_hi(r);
    }
    __device__ static void fma(const Raw &r, unsigned short v, float *acc) {
        fma_bf16x2(r, v, acc[0], acc[1]);
    }
    __device__ static void dot(const Raw &b, const Raw &f, float &d) { dot_bf16x2(b, f, d); }
};
template <>
struct Vec<uint16_t, 2> {
    static constexpr int E = 1;
    using Raw = unsigned short;
    __device__ static Raw raw(const uint16_t *p) { return __ldg(reinterpret_cast<const unsigned short *>(p)); }
    __device__ static float at(const Raw &r, int) { return __uint_as_float(static_cast<unsigned>(r) << 16); }
    __device__ static void load(const uint16_t *p, float *o) { o[0] = at(raw(p), 0); }
    __device__ static void fma(const Raw &r, unsigned short v, float *acc) { fma_bf16x1(r, v, acc[0]); }
    __device__ static void dot(const Raw &b, const Raw &f, float &d) { fma_bf16x1(b, f, d); }
};

// v[0..E) rounded to bf16 (nearest even) and stored at p, in whole vectors of up to 16 bytes
// (p aligned to min(2E, 16) bytes): the bf16 form of an fp32 output row segment. relu: negative
// values are stored as 0 first (the epilogue of a layer followed by a ReLU).
__device__ __forceinline__ unsigned pack_bf16x2(float lo, float hi) {
    return static_cast<unsigned>(f32_to_bf16(lo)) | (static_cast<unsigned>(f32_to_bf16(hi)) << 16);
}
template <int E>
__device__ __forceinline__ void store_bf16(uint16_t *p, const float *vin, bool relu = false) {
    float v[E];
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = relu_if(vin[i], relu);
    if constexpr (E % 8 == 0) {
#pragma unroll
        for (int i = 0; i < E; i += 8)
            *reinterpret_cast<uint4 *>(p + i) =
                make_uint4(pack_bf16x2(v[i], v[i + 1]), pack_bf16x2(v[i + 2], v[i + 3]),
                           pack_bf16x2(v[i + 4], v[i + 5]), pack_bf16x2(v[i + 6], v[i + 7]));
    } else if constexpr (E == 4) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]));
    } else if constexpr (E == 2) {
        *reinterpret_cast<unsigned *>(p) = pack_bf16x2(v[0], v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < E; ++i) p[i] = f32_to_bf16(v[i]);
    }
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

}  // namespace
}  // namespace as
