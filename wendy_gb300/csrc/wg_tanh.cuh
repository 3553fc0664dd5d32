// wg_tanh.cuh -- tanh on the integer pipes.
//
// FP64 issue is the scarce resource on GB300 (about 1/60 of the integer
// rate), and tanh(x / h) of the pulsed external force cost about 30 FP64
// instructions per sheet and force evaluation: as much time as the rest of
// the fused sub-step.  Here it is evaluated in 64-bit fixed point instead,
// with a handful of single-precision and conversion instructions:
//
//   tanh(a) = (1 - E) / (1 + E),  E = exp(-2a) = 2^-t,  t = 2 a log2(e),
//   t = k + j/64 + r  (k integer, 0 <= j < 64, 0 <= r < 1/64),
//   2^-t = 2^-k * 2^-(j/64) * exp(-r ln 2),
//
// 2^-(j/64) from a table, exp(-u) (u = r ln 2 < 0.0109) from its Taylor
// series to degree 7 (remainder below u^8/8! < 2e-21), and the quotient from
// a single-precision reciprocal refined by two Newton-Raphson steps.  t is
// formed from the full product of the 53-bit mantissa (one truncation, 2^-58
// in t, 2^-59.5 in the result); the other fixed-point quantities carry 62
// fractional bits and add a few 2^-62 truncations, so the absolute error
// before the final rounding to double is below 2^-57 for every finite input.  |y| < 2^-27 returns y
// (tanh(y) rounds to y there), |y| >= 20 returns +-1 (tanh(20) = 1 - 8.5e-18
// rounds to 1), NaN returns itself.
//
// The constants are round(2^62 2^(-j/64)), round(2^62 / n!), round(2^64 ln 2)
// and round(2^61 2 log2(e)), computed with 60-digit decimal arithmetic; the
// CPU tests recompute them the same way and compare.
#pragma once
#include <cstdint>

namespace wg {
namespace tanh_fx {

static __device__ const uint64_t kExp2Tab[64] __align__(128) = {
    0x4000000000000000ull, 0x3f4f83033d21b05dull, 0x3ea0ecb6dc8a80cfull, 0x3df437dcc2b44eeeull,
    0x3d495f454921b30bull, 0x3ca05dcf167fec4eull, 0x3bf92e66f736bd73ull, 0x3b53cc07b6650ae1ull,
    0x3ab031b9f7490e4cull, 0x3a0e5a940f12f71aull, 0x396e41b9df20d22aull, 0x38cfe25cafa29694ull,
    0x383337bb0aa53844ull, 0x37983d209783a449ull, 0x36feede5f6bc8dd5ull, 0x366745709e2bf5edull,
    0x35d13f32b5a75abdull, 0x353cd6aaf3fb7e88ull, 0x34aa07647c4ab917ull, 0x3418ccf6bbcac965ull,
    0x3389230547e12039ull, 0x32fb053fbc9c9f17ull, 0x326e6f619b8bc9e9ull, 0x31e35d322aee6c57ull,
    0x3159ca845541b6b7ull, 0x30d1b3368925d902ull, 0x304b1332999c2516ull, 0x2fc5e66d9e9cc421ull,
    0x2f4228e7d6030db0ull, 0x2ebfd6ac84cf917full, 0x2e3eebd1d8bee7baull, 0x2dbf6478ca345de4ull,
    0x2d413cccfe779921ull, 0x2cc47104aa444922ull, 0x2c48fd6074ab0964ull, 0x2bcede2b5a4290ddull,
    0x2b560fba90a852b2ull, 0x2ade8e6d6a4fb4ceull, 0x2a6856ad3a9f03beull, 0x29f364ed3a594d5aull,
    0x297fb5aa6c544e3bull, 0x290d456b8279a028ull, 0x289c10c0c3125a06ull, 0x282c1443ee5c53f1ull,
    0x27bd4c982468446bull, 0x274fb669cb3fedd4ull, 0x26e34e6e7553954eull, 0x26781164c82dfe99ull,
    0x260dfc14636e2a5cull, 0x25a50b4dc8061680ull, 0x253d3bea3fbdc258ull, 0x24d68acbc4f9ba4bull,
    0x2470f4dceac470ceull, 0x240c7710c519ac77ull, 0x23a90e62d17354f0ull, 0x2346b7d6df96ea79ull,
    0x22e57078faa2f5baull, 0x2285355d525bbf67ull, 0x222603a024b6a14aull, 0x21c7d865a7a34404ull,
    0x216ab0d9f3121ec5ull, 0x210e8a30eb379012ull, 0x20b361a62b0ae876ull, 0x2059347cef00c1ddull,
};
// round(2^62 / n!), n = 0 .. 7
__host__ __device__ constexpr uint64_t inv_fact_q62(int n) {
  return n <= 1   ? 0x4000000000000000ull
         : n == 2 ? 0x2000000000000000ull
         : n == 3 ? 0x0aaaaaaaaaaaaaabull
         : n == 4 ? 0x02aaaaaaaaaaaaabull
         : n == 5 ? 0x0088888888888889ull
         : n == 6 ? 0x0016c16c16c16c17ull
                  : 0x0003403403403403ull;
}
constexpr uint64_t kLn2Q64 = 0xb17217f7d1cf79acull;
constexpr uint64_t kTwoLog2eQ61 = 0x5c551d94ae0bf85eull;

// (a b) >> 62 for a b < 2^126
__device__ __forceinline__ uint64_t mul62(uint64_t a, uint64_t b) {
  return (__umul64hi(a, b) << 2) | ((a * b) >> 62);
}

}  // namespace tanh_fx

__device__ __forceinline__ double tanh_fixed(double y) {
  using namespace tanh_fx;
  const uint64_t bits = (uint64_t)__double_as_longlong(y);
  const uint64_t sign = bits & 0x8000000000000000ull;
  const uint64_t abits = bits ^ sign;
  if (abits < 0x3e40000000000000ull) return y;  // |y| < 2^-27, +-0, subnormals
  if (abits >= 0x4034000000000000ull) {          // |y| >= 20, +-inf, NaN
    if (abits > 0x7ff0000000000000ull) return y;
    return __longlong_as_double((long long)(sign | 0x3ff0000000000000ull));
  }
  // |y| = m 2^(e - 52); t = 2 |y| log2(e) with 58 fractional bits (t < 58),
  // from the full 117-bit product m L and one truncation:
  // t 2^58 = m L 2^(e - 52 - 61 + 58) = (m L) >> (55 - e)
  const int e = (int)(abits >> 52) - 1023;  // -27 .. 4
  const uint64_t m = (abits & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const uint64_t plo = m * kTwoLog2eQ61, phi = __umul64hi(m, kTwoLog2eQ61);
  const int s = 55 - e;  // 51 .. 82
  const uint64_t T = s >= 64 ? (phi >> (s - 64)) : ((phi << (64 - s)) | (plo >> s));
  const int k = (int)(T >> 58);
  const int j = (int)(T >> 52) & 63;
  const uint64_t rq = T & 0x000fffffffffffffull;  // r 2^58
  // u = r ln 2 with 62 fractional bits; exp(-u) by Horner, every partial
  // sum positive
  const uint64_t U = __umul64hi(rq << 4, kLn2Q64);
  uint64_t Q = inv_fact_q62(7);
#pragma unroll
  for (int n = 6; n >= 0; --n) Q = inv_fact_q62(n) - mul62(U, Q);
  const uint64_t E = mul62(__ldg(&kExp2Tab[j]), Q) >> k;
  const uint64_t N = (1ull << 62) - E;  // 1 - E
  const uint64_t D = (1ull << 62) + E;  // 1 + E, in (1, 2)
  // 1 / D: single-precision reciprocal (24 bits), two Newton-Raphson steps
  const float rf = __frcp_rn(__ull2float_rn(D) * 2.168404344971009e-19f);  // D 2^-62
  uint64_t R = __float2ull_rn(rf * 4.611686018427388e18f);                 // 2^62 / D
  R = mul62(R, (1ull << 63) - mul62(D, R));
  R = mul62(R, (1ull << 63) - mul62(D, R));
  const uint64_t Tq = mul62(N, R);  // tanh(a) 2^62, in (2^35, 2^62)
  // to double, rounding to nearest
  const int p = 63 - __clzll((long long)Tq);  // leading bit
  uint64_t mant;
  int be = p + 961;                            // biased exponent of 2^(p - 62)
  if (p > 52) {
    const int q = p - 52;
    mant = (Tq + (1ull << (q - 1))) >> q;
    if (mant >> 53) {
      mant >>= 1;
      ++be;
    }
  } else {
    mant = Tq << (52 - p);
  }
  return __longlong_as_double(
      (long long)(sign | ((uint64_t)be << 52) | (mant & 0x000fffffffffffffull)));
}

}  // namespace wg
