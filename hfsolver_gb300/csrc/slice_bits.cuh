// Integer-only pieces of the exact bf16 slicing (tcgemm.cu), shared by the
// device kernels and host-side checks.
//
// A row with exponent e (|x| < 2^e for every element) is scaled to the integer
// Y = round(|x| 2^(42 - e)) < 2^42 (+1 by rounding), cut into six 7-bit digits
// Y = sum_t d_t 2^(7 (5 - t)) (d_0 may reach 128), and each digit is stored as
// the bf16 value sign(x) d_t.  GB300 runs 64-bit conversions on its narrow
// FP64 pipe, so everything here is integer arithmetic, except for one packed
// bf16 subtraction per two digits: the bit pattern 0x4300 | d is the bf16
// value 128 + d for 0 <= d <= 128 (the digit lands in the mantissa, or for
// d = 128 carries into the exponent), and subtracting 128 leaves exactly d.
//
// The epilogue's conversion back, RN((double) S) 2^E for the int64 sum S of
// the digit products, is done the same way: the double's fields are assembled
// from the integer's leading bit and a round-to-nearest-even of the bits below
// the 53rd, so the FP64 pipe is not used for the output either.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define HF_HD __host__ __device__ __forceinline__
#else
#define HF_HD inline
#endif

namespace hfgpu {

constexpr int SLICE_NSL = 6, SLICE_BITS = 7;

HF_HD int clz64(uint64_t v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// round(|x| 2^(42 - e)) from the bits of x (0 for zero and subnormal x)
HF_HD uint64_t scaled_magnitude(uint64_t bits, int e)
{
    const int ex = (int)((bits >> 52) & 0x7FF);
    uint64_t Y = 0;
    if (ex != 0) {
        const uint64_t m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = ex - 1075 + SLICE_NSL * SLICE_BITS - e;  // |x| < 2^e gives sh < -10
        if (sh >= 0)
            Y = m << sh;
        else if (sh > -63)
            Y = (m + (1ull << (-sh - 1))) >> (-sh);
    }
    return Y;
}

// digit t (0: most significant) of Y
HF_HD uint32_t digit(uint64_t Y, int t)
{
    const int shift = SLICE_BITS * (SLICE_NSL - 1 - t);
    return (uint32_t)(Y >> shift) & (t == 0 ? 0xFFFFFFFFu : ((1u << SLICE_BITS) - 1));
}

// plane t of two elements before the subtraction: bf16 patterns of 128 + d
// (element 0 in the low half)
HF_HD uint32_t digit_word(uint64_t Y0, uint64_t Y1, int t)
{
    return 0x43004300u | digit(Y0, t) | (digit(Y1, t) << 16);
}

// sign bits of two elements, in place for the packed bf16 pair
HF_HD uint32_t sign_word(uint64_t bits0, uint64_t bits1)
{
    return (uint32_t)(bits0 >> 63) << 15 | (uint32_t)(bits1 >> 63) << 31;
}

// RN((double) S) 2^E assembled from integer fields.  ok = false when the result
// would be subnormal or overflow (the caller then uses the FP64 unit).
HF_HD uint64_t scaled_int_to_double_bits(long long S, int E, bool& ok)
{
    ok = true;
    if (S == 0) return 0;
    const uint64_t sign = S < 0 ? 1ull : 0ull;
    const uint64_t m = sign ? (uint64_t)0 - (uint64_t)S : (uint64_t)S;
    int msb = 63 - clz64(m);
    uint64_t mant;
    if (msb <= 52) {
        mant = m << (52 - msb);
    } else {
        const int sh = msb - 52;
        const uint64_t rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        mant = m >> sh;
        if (rem > half || (rem == half && (mant & 1ull))) {
            ++mant;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                ++msb;
            }
        }
    }
    const int ef = msb + E + 1023;
    if (ef <= 0 || ef >= 2047) {
        ok = false;
        return 0;
    }
    return sign << 63 | (uint64_t)ef << 52 | (mant & ((1ull << 52) - 1));
}

}  // namespace hfgpu
