/*
 * Portable stand-in for the SSE1 intrinsics header, used ONLY to compile the
 * reference CPU code (oracle/_ref) with g++ on x86-64 and on aarch64.
 *
 * Test infrastructure: nothing in the shipped library includes this file.
 *
 * Why a class type: the reference declares global operator overloads on
 * __m128 (KinectFission/kifi/util/math.h:157-179, :779-871).  GCC treats the
 * native __m128 as a built-in vector type and rejects such overloads; with a
 * class type they are ordinary, legal overloads, so the reference's math.h
 * compiles unmodified and its operators route through the functions below.
 *
 * Semantics: every lane operation is one IEEE-754 single-precision operation
 * with round-to-nearest and no denormal flushing, which is what SSE1 does
 * under the default MXCSR.  Build with -ffp-contract=off so that no
 * multiply/add pair is fused on targets that have FMA.  Comparisons return an
 * all-ones / all-zeros lane mask like CMPPS (ordered for lt/le/gt/ge/eq,
 * unordered-true for neq).
 */
#ifndef KIFI_ORACLE_SHIM_XMMINTRIN_H
#define KIFI_ORACLE_SHIM_XMMINTRIN_H

#include <cmath>
#include <cstdint>
#include <cstring>

struct alignas(16) __m128 {
    float f[4];
};

namespace kifi_sse_shim {
inline float mask_lane(bool b) {
    std::uint32_t u = b ? 0xffffffffu : 0u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
inline std::uint32_t bits(float x) {
    std::uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
}
inline float from_bits(std::uint32_t u) {
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
}  // namespace kifi_sse_shim

#define KIFI_SHIM_LANEWISE(name, expr)                       \
    static inline __m128 name(__m128 a, __m128 b) {          \
        __m128 r;                                            \
        for (int i = 0; i < 4; ++i) {                        \
            float x = a.f[i], y = b.f[i];                    \
            r.f[i] = (expr);                                 \
        }                                                    \
        return r;                                            \
    }

KIFI_SHIM_LANEWISE(_mm_add_ps, x + y)
KIFI_SHIM_LANEWISE(_mm_sub_ps, x - y)
KIFI_SHIM_LANEWISE(_mm_mul_ps, x * y)
KIFI_SHIM_LANEWISE(_mm_div_ps, x / y)
KIFI_SHIM_LANEWISE(_mm_cmpeq_ps, kifi_sse_shim::mask_lane(x == y))
KIFI_SHIM_LANEWISE(_mm_cmpneq_ps, kifi_sse_shim::mask_lane(!(x == y)))
KIFI_SHIM_LANEWISE(_mm_cmplt_ps, kifi_sse_shim::mask_lane(x < y))
KIFI_SHIM_LANEWISE(_mm_cmple_ps, kifi_sse_shim::mask_lane(x <= y))
KIFI_SHIM_LANEWISE(_mm_cmpgt_ps, kifi_sse_shim::mask_lane(x > y))
KIFI_SHIM_LANEWISE(_mm_cmpge_ps, kifi_sse_shim::mask_lane(x >= y))
KIFI_SHIM_LANEWISE(_mm_and_ps, kifi_sse_shim::from_bits(kifi_sse_shim::bits(x) & kifi_sse_shim::bits(y)))
KIFI_SHIM_LANEWISE(_mm_or_ps, kifi_sse_shim::from_bits(kifi_sse_shim::bits(x) | kifi_sse_shim::bits(y)))

#undef KIFI_SHIM_LANEWISE

static inline __m128 _mm_sqrt_ps(__m128 a) {
    __m128 r;
    for (int i = 0; i < 4; ++i) r.f[i] = std::sqrt(a.f[i]);
    return r;
}

static inline int _mm_movemask_ps(__m128 a) {
    int m = 0;
    for (int i = 0; i < 4; ++i) m |= (int)(kifi_sse_shim::bits(a.f[i]) >> 31) << i;
    return m;
}

static inline __m128 _mm_load_ps(float const* p) {
    __m128 r;
    std::memcpy(r.f, p, 16);
    return r;
}
static inline __m128 _mm_loadu_ps(float const* p) { return _mm_load_ps(p); }
static inline __m128 _mm_load_ss(float const* p) {
    __m128 r = {{*p, 0.0f, 0.0f, 0.0f}};
    return r;
}
static inline __m128 _mm_set1_ps(float s) {
    __m128 r = {{s, s, s, s}};
    return r;
}
/* Argument order follows SSE: the LAST argument is lane 0. */
static inline __m128 _mm_set_ps(float w, float z, float y, float x) {
    __m128 r = {{x, y, z, w}};
    return r;
}
static inline __m128 _mm_setzero_ps() { return _mm_set1_ps(0.0f); }

#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))
static inline __m128 kifi_shim_shuffle(__m128 a, __m128 b, int imm) {
    __m128 r = {{a.f[imm & 3], a.f[(imm >> 2) & 3], b.f[(imm >> 4) & 3], b.f[(imm >> 6) & 3]}};
    return r;
}
#define _mm_shuffle_ps(a, b, imm) kifi_shim_shuffle((a), (b), (imm))

static inline void _mm_store_ps(float* p, __m128 a) { std::memcpy(p, a.f, 16); }
static inline void _mm_storeu_ps(float* p, __m128 a) { std::memcpy(p, a.f, 16); }
static inline void _mm_store_ss(float* p, __m128 a) { *p = a.f[0]; }

#endif
