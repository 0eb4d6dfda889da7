// hcore-gb300: FP64-accurate products on the bf16 tensor cores, the pieces
// shared by the kernels that use them (the rebuild, hc_rebuild_tc.cu, and the
// blocked QR's trailing update, hc_qr_tc.cu).
//
// A value x of a row or column with common scale 2^E becomes the integer
// X = round(x 2^(55-E)), |X| <= 2^55, written as seven balanced base-256
// digits in [-128, 128] (each exact in bf16): the error-free splitting of
// Ozaki, Ogita, Oishi and Rump (2012) in the fixed-point form of Mukunoki,
// Ozaki, Ogita and Imamura (2020).  A digit product is at most 2^14, so a sum
// of up to 1024 of them is an integer below 2^24, which an FP32 accumulator
// holds exactly.  Digit products of equal weight d = i + l share one tensor-
// memory accumulator ("plane"); planes 0..7 are kept, the dropped ones are
// below 2^-61 of the largest product.  The planes are combined exactly in
// 64-bit integers and the FP64 result is assembled from the integer.
#pragma once
#include <stdint.h>

#include "hc_tc.cuh"

namespace hc {
namespace dg {

constexpr int kPlanes = 8;                      // digit-product weights d = 0..7
constexpr long long kTcWaitCycles = 1LL << 30;  // bounded MMA waits: about half a second

__device__ __forceinline__ int exp_field(double x) {
    return (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7FF;
}

// X = round(x 2^(55 - E)) for |x| < 2^E (|X| < 2^55), from the bits alone.
__device__ __forceinline__ long long fixed55(double x, int E) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ef = (int)(b >> 52) & 0x7FF;
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int e2;
    if (ef == 0) {
        e2 = -1074;
    } else {
        m |= 1ull << 52;
        e2 = ef - 1075;
    }
    const int sh = e2 + 55 - E;
    long long X;
    if (sh >= 0) X = (long long)(m << sh);
    else if (sh > -64) X = (long long)((m + (1ull << (-sh - 1))) >> (-sh));
    else X = 0;
    return (b >> 63) ? -X : X;
}

__device__ __forceinline__ uint32_t pack_bf16(uint32_t lo, uint32_t hi) {
    return __byte_perm(lo, hi, 0x7632);
}

// Two adjacent planes combined exactly, q = acc_2m 2^8 + acc_2m+1 (|q| <
// 2^33), added as q 2^(88 - 16 m - S); a right shift rounds to nearest, so
// the few bits dropped below the combined value's last place do not bias it.
template <int S, int PM>
__device__ __forceinline__ long long pair_term(float v0, float v1) {
    constexpr int sh = 88 - 16 * PM - S;
    const long long q = (long long)__float2int_rn(v0) * 256 + (long long)__float2int_rn(v1);
    if constexpr (sh >= 0) return q * (1LL << sh);
    else return (q + (1LL << (-sh - 1))) >> (-sh);
}

// add the eight planes of 8 columns (taddr: lane base + first column; plane
// d sits d * stride columns further) into the running sums
template <int S, int PM>
__device__ __forceinline__ void add_pair(long long (&acc)[8], uint32_t taddr, int stride) {
    float v0[8], v1[8];
    tc::tmem_ld8(taddr + (2 * PM) * stride, v0);
    tc::tmem_ld8(taddr + (2 * PM + 1) * stride, v1);
    tc::tmem_ld_wait();
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] += pair_term<S, PM>(v0[e], v1[e]);
}
template <int S>
__device__ __forceinline__ void combine_planes(long long (&acc)[8], uint32_t taddr, int stride) {
    add_pair<S, 0>(acc, taddr, stride);
    add_pair<S, 1>(acc, taddr, stride);
    add_pair<S, 2>(acc, taddr, stride);
    add_pair<S, 3>(acc, taddr, stride);
}

// T 2^p as an FP64 value, rounded to nearest even, by integer instructions
// only (the FP64 pipe is the busy one); ok = false when the result leaves the
// normal range, and the caller converts with FP64 arithmetic instead.
__device__ __forceinline__ double i64_times_pow2(long long T, int p, bool &ok) {
    if (T == 0) {
        ok = true;
        return 0.0;
    }
    const unsigned long long sgn = (unsigned long long)T & 0x8000000000000000ull;
    unsigned long long m = T < 0 ? 0ull - (unsigned long long)T : (unsigned long long)T;
    const int lz = __clzll((long long)m);
    m <<= lz;                                    // leading one at bit 63
    int e = 63 - lz + p;
    unsigned long long mant = m >> 11;           // 53 bits
    const unsigned rem = (unsigned)(m & 0x7FFu);
    mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    if (mant >> 53) {
        mant >>= 1;
        ++e;
    }
    ok = e >= -1022 && e <= 1023;
    return __longlong_as_double(
        (long long)(sgn | ((unsigned long long)(e + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// x 2^p for any p a product of two FP64 values can need (exact unless the
// result is subnormal)
__device__ __forceinline__ double scale2(double x, int p) {
    const int p1 = p / 2, p2 = p - p1;
    if (p >= -1022 && p <= 1023) return x * __longlong_as_double((long long)(p + 1023) << 52);
    return (x * __longlong_as_double((long long)(p1 + 1023) << 52)) *
           __longlong_as_double((long long)(p2 + 1023) << 52);
}

// Seven balanced base-256 digits of X (|X| <= 2^55) as FP32 bit patterns,
// without a data-dependent loop: Z = X + B with B = 128 (256^6 + ... + 1) is
// non-negative, digit i is byte 6 - i of Z minus 128 (the top one, Z >> 48,
// may be 256).  One byte permute moves a byte into the mantissa of 2^23 and
// one FP32 add removes 2^23 + 128, exactly.
__device__ __forceinline__ void digits7_fast(long long X, uint32_t (&f)[7]) {
    const unsigned long long z = (unsigned long long)X + 0x0080808080808080ull;
    const uint32_t lo = (uint32_t)z, hi = (uint32_t)(z >> 32);
    const float c = 8388736.0f;  // 2^23 + 128
    f[6] = __float_as_uint(__uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7540)) - c);
    f[5] = __float_as_uint(__uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7541)) - c);
    f[4] = __float_as_uint(__uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7542)) - c);
    f[3] = __float_as_uint(__uint_as_float(__byte_perm(lo, 0x4B000000u, 0x7543)) - c);
    f[2] = __float_as_uint(__uint_as_float(__byte_perm(hi, 0x4B000000u, 0x7540)) - c);
    f[1] = __float_as_uint(__uint_as_float(__byte_perm(hi, 0x4B000000u, 0x7541)) - c);
    f[0] = __float_as_uint(__uint_as_float(0x4B000000u | (hi >> 16)) - c);
}

// Seven 16-byte core-matrix rows of zeros (a padding row of every plane).
__device__ __forceinline__ void zero8(unsigned char *dst, int slice_stride) {
#pragma unroll
    for (int s = 0; s < 7; ++s)
        *reinterpret_cast<uint4 *>(dst + s * slice_stride) = make_uint4(0, 0, 0, 0);
}

// Slice eight values that share the scale 2^E (consecutive along K) into
// seven 16-byte core-matrix rows, one per digit plane, slice_stride apart;
// with dst2 != nullptr the same rows also go to a second operand buffer.
__device__ __forceinline__ void slice8(const double (&x)[8], int E, unsigned char *dst,
                                       int slice_stride, unsigned char *dst2 = nullptr,
                                       int slice_stride2 = 0) {
    uint32_t w[7][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t f0[7], f1[7];
        digits7_fast(fixed55(x[2 * q], E), f0);
        digits7_fast(fixed55(x[2 * q + 1], E), f1);
#pragma unroll
        for (int s = 0; s < 7; ++s) w[s][q] = pack_bf16(f0[s], f1[s]);
    }
#pragma unroll
    for (int s = 0; s < 7; ++s)
        *reinterpret_cast<uint4 *>(dst + s * slice_stride) =
            make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    if (dst2) {
#pragma unroll
        for (int s = 0; s < 7; ++s)
            *reinterpret_cast<uint4 *>(dst2 + s * slice_stride2) =
                make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}


// Issue the MMAs of one pass: planes d = 0..7 (accumulator d at tensor-memory
// column tbase + d * pstride) from seven A digit slices (a_stride bytes
// apart, row-group stride a_sbo) and B digit slices (b_stride apart, b_sbo),
// one MMA (M = 128, K = 16) per A slice i, K step and piece of planes, whose
// B operand is the run of consecutive B slices d0 - i .. d1 - i (an eighth,
// zero B slice ends the run), so the product with B slice l lands in plane
// i + l.  A piece spans at most 256 columns; the first MMAs (i = 0, K step 0)
// cover every plane and start the accumulators.  One thread calls this; the
// mbarrier receives one arrival when the MMAs are done.
__device__ __forceinline__ void issue_planes(uint32_t tbase, uint64_t *mbar, uint32_t a0,
                                             int a_stride, uint32_t a_sbo, uint32_t b0,
                                             int b_stride, uint32_t b_sbo, int ksteps,
                                             int pstride) {
    const int per = 256 / pstride;
#pragma unroll 1
    for (int i = 0; i < 7; ++i) {
        const uint64_t da = tc::make_desc(a0 + i * a_stride, tc::kLbo, a_sbo);
#pragma unroll 1
        for (int d0 = i; d0 < kPlanes; d0 += per) {
            const int d1 = d0 + per < kPlanes ? d0 + per : kPlanes;
            const uint64_t db = tc::make_desc(b0 + (d0 - i) * b_stride, tc::kLbo, b_sbo);
            const uint32_t id = tc::idesc_bf16_f32(128, (d1 - d0) * pstride);
#pragma unroll 1
            for (int s = 0; s < ksteps; ++s)
                tc::mma_bf16(tbase + d0 * pstride, da + 16 * s, db + 16 * s, id, i > 0 || s > 0);
        }
    }
    tc::mma_commit(mbar);
}

}  // namespace dg
}  // namespace hc
