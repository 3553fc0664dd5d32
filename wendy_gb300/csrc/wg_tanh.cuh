// wg_tanh.cuh -- tanh on the integer pipes.
//
// FP64 issue is the scarce resource on GB300 (about 1/60 of the integer
// rate), and tanh(x / h) of the pulsed external force cost about 30 FP64
// instructions per sheet and force evaluation: as much time as the rest of
// the fused sub-step.  Here it is evaluated in 64-bit fixed point instead,
// with a handful of single-precision and conversion instructions:
//
//   tanh(a) = (1 - E) / (1 + E),  E = exp(-2a) = 2^-t,  t = 2 a log2(e),
//   t = k + j/256 + r  (k integer, 0 <= j < 256, 0 <= r < 1/256),
//   2^-t = 2^-k * 2^-(j/256) * exp(-r ln 2),
//
// 2^-(j/256) from a 2 KB table, exp(-u) (u = r ln 2 < 0.0028) from its
// Taylor series to degree 5 (remainder below u^6/6! < 7e-19), and the quotient from
// a single-precision reciprocal refined by two Newton-Raphson steps.  t is
// formed from the full product of the 53-bit mantissa (one truncation, 2^-58
// in t, 2^-59.5 in the result); the other fixed-point quantities carry 62
// fractional bits and add a few 2^-62 truncations, so the absolute error
// before the final rounding to double is below 2^-57 for every finite input.  |y| < 2^-27 returns y
// (tanh(y) rounds to y there), |y| >= 20 returns +-1 (tanh(20) = 1 - 8.5e-18
// rounds to 1), NaN returns itself.
//
// The constants are round(2^62 2^(-j/256)), round(2^62 / n!), round(2^64 ln 2)
// and round(2^61 2 log2(e)), computed with 60-digit decimal arithmetic; the
// CPU tests recompute them the same way and compare.
//
// The force kernels do not call this per sheet: tanh_q62 fills, once per
// device, a table of degree-5 Taylor polynomials on cells of width 2^-10
// (tanh_tab, at the end of this file), which costs a fraction of it.
#pragma once
#include <cstdint>

namespace wg {
namespace tanh_fx {

static __device__ const uint64_t kExp2Tab[256] __align__(128) = {
    0x4000000000000000ull, 0x3fd3b2d65447b229ull, 0x3fa784571ee3e213ull, 0x3f7b746d25aa27cdull,
    0x3f4f83033d21b05dull, 0x3f23b004487911efull, 0x3ef7fb5b397c2712ull, 0x3ecc64f31089f0fdull,
    0x3ea0ecb6dc8a80cfull, 0x3e759291bae4e7cdull, 0x3e4a566ed7752e9dull, 0x3e1f38396c825367ull,
    0x3df437dcc2b44eeeull, 0x3dc95544310a208eull, 0x3d9e905b1ccfe11bull, 0x3d73e90cf994dca4ull,
    0x3d495f454921b30bull, 0x3d1ef2ef9b6e7f78ull, 0x3cf4a3f78e990697ull, 0x3cca7248cedaeba7ull,
    0x3ca05dcf167fec4eull, 0x3c7666762ddc2330ull, 0x3c4c8c29eb425142ull, 0x3c22ced632fa2ddbull,
    0x3bf92e66f736bd73ull, 0x3bcfaac8380caf1bull, 0x3ba643e60368c097ull, 0x3b7cf9ac75062924ull,
    0x3b53cc07b6650ae1ull, 0x3b2abae3fec0ead0ull, 0x3b01c62d93072f77ull, 0x3ad8edd0c5cda610ull,
    0x3ab031b9f7490e4cull, 0x3a8791d59543ac9full, 0x3a5f0e101b13e316ull, 0x3a36a6561192d0abull,
    0x3a0e5a940f12f71aull, 0x39e62ab6b756e730ull, 0x39be16aabb87f389ull, 0x39961e5cda2ce9c6ull,
    0x396e41b9df20d22aull, 0x394680aea389b5a0ull, 0x391edb280dcf6a23ull, 0x38f7511311926586ull,
    0x38cfe25cafa29694ull, 0x38a88ef1f5f64489ull, 0x388156bfffa0f4daull, 0x385a39b3f4ca5749ull,
    0x383337bb0aa53844ull, 0x380c50c28366798aull, 0x37e584b7ae3c1108ull, 0x37bed387e7440dfcull,
    0x37983d209783a449ull, 0x3771c16f34de3dfcull, 0x374b6061420c9308ull, 0x372519e44e93c724ull,
    0x36feede5f6bc8dd5ull, 0x36d8dc53e38a5495ull, 0x36b2e51bcab2731cull, 0x368d082b6e9361c1ull,
    0x366745709e2bf5edull, 0x36419cd93512a4a7ull, 0x361c0e531b6ccb21ull, 0x35f699cc45e5fd5aull,
    0x35d13f32b5a75abdull, 0x35abfe74784ee8bfull, 0x3586d77fa7e6f382ull, 0x3561ca426add7462ull,
    0x353cd6aaf3fb7e88ull, 0x3517fca7825cb158ull, 0x34f33c266166b0deull, 0x34ce9515e8c0a415ull,
    0x34aa07647c4ab917ull, 0x348593008c15af2bull, 0x346137d8945a66b2ull, 0x343cf5db1d7176e3ull,
    0x3418ccf6bbcac965ull, 0x33f4bd1a0fe53badull, 0x33d0c633c6464630ull, 0x33ace8329771a957ull,
    0x3389230547e12039ull, 0x3365769aa7fc1911ull, 0x3341e2e1940f7374ull, 0x331e67c8f4454439ull,
    0x32fb053fbc9c9f17ull, 0x32d7bb34ece165f2ull, 0x32b4899790a41dd3ull, 0x32917056bf31c989ull,
    0x326e6f619b8bc9e9ull, 0x324b86a7545fc3b3ull, 0x3228b61723ff8b11ull, 0x3205fda0505914adull,
    0x31e35d322aee6c57ull, 0x31c0d4bc10cdb147ull, 0x319e642d6a8917deull, 0x317c0b75ac2ef0f6ull,
    0x3159ca845541b6b7ull, 0x3137a148f0b01eebull, 0x31158fb314cd32cdull, 0x30f395b263486c57ull,
    0x30d1b3368925d902ull, 0x30afe82f3eb641f2ull, 0x308e348c478f599dull, 0x306c983d7283eecdull,
    0x304b1332999c2516ull, 0x3029a55ba20db2a3ull, 0x30084ea87c34236cull, 0x2fe70f09238921beull,
    0x2fc5e66d9e9cc421ull, 0x2fa4d4c5ff0de08eull, 0x2f83da02618264f9ull, 0x2f62f612ed9fb521ull,
    0x2f4228e7d6030db0ull, 0x2f2172715839ec9aull, 0x2f00d29fbcba7ec3ull, 0x2ee0496356dc12dcull,
    0x2ebfd6ac84cf917full, 0x2e9f7a6baf97fa82ull, 0x2e7f34914b02e77bull, 0x2e5f050dd5a11370ull,
    0x2e3eebd1d8bee7baull, 0x2e1ee8cde85d0e0dull, 0x2dfefbf2a329079full, 0x2ddf2530b275c97aull,
    0x2dbf6478ca345de4ull, 0x2d9fb9bba8ec8ae4ull, 0x2d8024ea17b57ddbull, 0x2d60a5f4ea2e7c34ull,
    0x2d413cccfe779921ull, 0x2d21e9633d2a7060ull, 0x2d02aba89952e610ull, 0x2ce3838e1067eb86ull,
    0x2cc47104aa444922ull, 0x2ca573fd791f6d29ull, 0x2c868c6999863f8full, 0x2c67ba3a3253fac2ull,
    0x2c48fd6074ab0964ull, 0x2c2a55cd9bede8f2ull, 0x2c0bc372edb81161ull, 0x2bed4641b9d6e198ull,
    0x2bcede2b5a4290ddull, 0x2bb08b2133172519ull, 0x2b924d14b28d6e04ull, 0x2b7423f750f40524ull,
    0x2b560fba90a852b2ull, 0x2b38104ffe0f9741ull, 0x2b1a25a92f8ffa4aull, 0x2afc4fb7c5899d7aull,
    0x2ade8e6d6a4fb4ceull, 0x2ac0e1bbd221a378ull, 0x2aa34994bb241d8aull, 0x2a85c5e9ed5a4e5eull,
    0x2a6856ad3a9f03beull, 0x2a4afbd07e9dddc7ull, 0x2a2db5459ecc8382ull, 0x2a1082fe8a63dc34ull,
    0x29f364ed3a594d5aull, 0x29d65b03b157fd57ull, 0x29b96533fbba1ac7ull, 0x299c83702f822883ull,
    0x297fb5aa6c544e3bull, 0x2962fbd4db6fadbbull, 0x294655e1afa7bcceull, 0x2929c3c3255da3b1ull,
    0x290d456b8279a028ull, 0x28f0dacd16646d1full, 0x28d483da3a00aee5ull, 0x28b840854fa463e8ull,
    0x289c10c0c3125a06ull, 0x287ff47f0973a862ull, 0x2863ebb2a1512db9ull, 0x2847f64e128d133eull,
    0x282c1443ee5c53f1ull, 0x28104586cf40486full, 0x27f48a0959003741ull, 0x27d8e1be38a2e994ull,
    0x27bd4c982468446bull, 0x27a1ca89dbc2e640ull, 0x27865b862751c908ull, 0x276aff7fd8d9e8aaull,
    0x274fb669cb3fedd4ull, 0x27348036e281dd33ull, 0x27195cda0bb0cb0bull, 0x26fe4c463cea9330ull,
    0x26e34e6e7553954eull, 0x26c86345bd10758full, 0x26ad8abf253fe193ull, 0x2692c4cdc7f459b3ull,
    0x26781164c82dfe99ull, 0x265d707751d4631eull, 0x2642e1f899b0626aull, 0x262865dbdd65fa65ull,
    0x260dfc14636e2a5cull, 0x25f3a4957b10d5ebull, 0x25d95f527c5eac24ull, 0x25bf2c3ec82b12e9ull,
    0x25a50b4dc8061680ull, 0x258afc72ee365d58ull, 0x2570ffa1b5b31ffcull, 0x255714cda21e2535ull,
    0x253d3bea3fbdc258ull, 0x252374eb2376dfb5ull, 0x2509bfc3eac7012eull, 0x24f01c683bbe52f0ull,
    0x24d68acbc4f9ba4bull, 0x24bd0ae23d9cea9full, 0x24a39c9f654c7e6bull, 0x248a3ff70428146bull,
    0x2470f4dceac470ceull, 0x2457bb44f225a275ull, 0x243e9322fbb92c4bull, 0x24257c6af150329bull,
    0x240c7710c519ac77ull, 0x23f38308719c9920ull, 0x23daa045f9b23971ull, 0x23c1cebd68804d48ull,
    0x23a90e62d17354f0ull, 0x23905f2a5038d680ull, 0x2377c10808b9a735ull, 0x235f33f0271438beull,
    0x2346b7d6df96ea79ull, 0x232e4cb06eba5ea5ull, 0x2315f271191bd377ull, 0x22fda90d2b778021ull,
    0x22e57078faa2f5baull, 0x22cd48a8e387840cull, 0x22b531914b1ca249ull, 0x229d2b269e625b92ull,
    0x2285355d525bbf67ull, 0x226d5029e40955e9ull, 0x22557b80d86397f7ull, 0x223db756bc556b1bull,
    0x222603a024b6a14aull, 0x220e6051ae467c75ull, 0x21f6cd5ffda635e4ull, 0x21df4abfbf53895bull,
    0x21c7d865a7a34404ull, 0x21b0764672bbd722ull, 0x21992456e48fee81ull, 0x2181e28bc8d90aa8ull,
    0x216ab0d9f3121ec5ull, 0x21538f363e723257ull, 0x213c7d958de7068aull, 0x21257beccc0fbf4cull,
    0x210e8a30eb379012ull, 0x20f7a856e5506c4dull, 0x20e0d653bbedbb8eull, 0x20ca141c783f1152ull,
    0x20b361a62b0ae876ull, 0x209cbee5eca96253ull, 0x20862bd0dcff097bull, 0x206fa85c23779815ull,
    0x2059347cef00c1ddull, 0x2042d028760501b5ull, 0x202c7b53f6666adbull, 0x201635f4b5797dacull,
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

// tanh(|y|) 2^62 for 2^-27 <= |y| < 20, |y| given by its bits; the absolute
// error is below 2^-57 (the bound stated above).
__device__ __forceinline__ uint64_t tanh_q62(uint64_t abits) {
  using namespace tanh_fx;
  // |y| = m 2^(e - 52); t = 2 |y| log2(e) with 58 fractional bits (t < 58),
  // from the full 117-bit product m L and one truncation:
  // t 2^58 = m L 2^(e - 52 - 61 + 58) = (m L) >> (55 - e)
  const int e = (int)(abits >> 52) - 1023;  // -27 .. 4
  const uint64_t m = (abits & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const uint64_t plo = m * kTwoLog2eQ61, phi = __umul64hi(m, kTwoLog2eQ61);
  const int s = 55 - e;  // 51 .. 82
  const uint64_t T = s >= 64 ? (phi >> (s - 64)) : ((phi << (64 - s)) | (plo >> s));
  const int k = (int)(T >> 58);
  const int j = (int)(T >> 50) & 255;
  const uint64_t rq = T & 0x0003ffffffffffffull;  // r 2^58
  // u = r ln 2 with 62 fractional bits; exp(-u) by Horner, every partial
  // sum positive
  const uint64_t U = __umul64hi(rq << 4, kLn2Q64);
  uint64_t Q = inv_fact_q62(5);
#pragma unroll
  for (int n = 4; n >= 0; --n) Q = inv_fact_q62(n) - mul62(U, Q);
  const uint64_t E = mul62(__ldg(&kExp2Tab[j]), Q) >> k;
  const uint64_t N = (1ull << 62) - E;  // 1 - E
  const uint64_t D = (1ull << 62) + E;  // 1 + E, in (1, 2)
  // 1 / D: single-precision reciprocal (24 bits), two Newton-Raphson steps
  const float rf = __frcp_rn(__ull2float_rn(D) * 2.168404344971009e-19f);  // D 2^-62
  uint64_t R = __float2ull_rn(rf * 4.611686018427388e18f);                 // 2^62 / D
  R = mul62(R, (1ull << 63) - mul62(D, R));
  R = mul62(R, (1ull << 63) - mul62(D, R));
  return mul62(N, R);  // tanh(a) 2^62, in (2^35, 2^62)
}

// Tq 2^-62 (0 < Tq < 2^62) to double, rounded to nearest, with the sign bit given.
__device__ __forceinline__ double q62_to_double(uint64_t Tq, uint64_t sign) {
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

__device__ __forceinline__ double tanh_fixed(double y) {
  const uint64_t bits = (uint64_t)__double_as_longlong(y);
  const uint64_t sign = bits & 0x8000000000000000ull;
  const uint64_t abits = bits ^ sign;
  if (abits < 0x3e40000000000000ull) return y;  // |y| < 2^-27, +-0, subnormals
  if (abits >= 0x4034000000000000ull) {          // |y| >= 20, +-inf, NaN
    if (abits > 0x7ff0000000000000ull) return y;
    return __longlong_as_double((long long)(sign | 0x3ff0000000000000ull));
  }
  return q62_to_double(tanh_q62(abits), sign);
}

// ---------------------------------------------------------------------------
// tanh from a table of Taylor polynomials.  The argument range [0, 20) is cut
// into cells of width 2^-10; cell i holds, in 2^62 fixed point, t = tanh(a_i)
// at a_i = i 2^-10 (from tanh_q62) and the Taylor coefficients about a_i,
//
//   tanh(a_i + D) = t + s D - t s D^2 + s (3t^2 - 1)/3 D^3
//                   + t s (2 - 3t^2)/3 D^4 + s (2 - 15t^2 + 15t^4)/15 D^5 + O(D^6),
//
// s = 1 - t^2 (the derivatives follow from t' = s, s' = -2ts).  With
// 0 <= D < 2^-10 the remainder is below 2^-64 (the Taylor coefficients of
// tanh are below 1), s is formed in fixed point and the higher coefficients
// in double (their rounding enters multiplied by D^2 <= 2^-20), and each
// Horner step is one signed high product with D 2^64, so the absolute error
// stays within that of tanh_q62 plus 2^-61.  The cell and D come from the
// argument's bits (D is exact up to one truncation of 2^-64).  Per argument
// this is some 35 integer instructions and three 16-byte loads, which hit
// in L1 for the sorted positions of a bucket or tile, against about 150
// instructions and two conversions on the FP64 pipe for tanh_fixed.  The
// table (20480 cells, 960 KB) is computed once per device by
// k_tanh_table; the result is a function of the argument alone, so every
// kernel that evaluates the force gives the same bits.
// ---------------------------------------------------------------------------
constexpr int kTanhCellBits = 10;
constexpr int kTanhCells = 20 << kTanhCellBits;
constexpr int kTanhRow = 6;  // t, then the coefficients of D .. D^5

// Row of cell i.
__device__ __forceinline__ void tanh_table_row(int i, long long* row) {
  const double a = (double)i * 0x1p-10;
  const uint64_t tq = i == 0 ? 0ull : tanh_q62((uint64_t)__double_as_longlong(a));
  const uint64_t s = (1ull << 62) - tanh_fx::mul62(tq, tq);
  const double td = (double)tq * 0x1p-62, sd = (double)s * 0x1p-62;
  const double t2 = td * td;
  row[0] = (long long)tq;
  row[1] = (long long)s;
  row[2] = __double2ll_rn(-td * sd * 0x1p62);
  row[3] = __double2ll_rn(sd * (3.0 * t2 - 1.0) / 3.0 * 0x1p62);
  row[4] = __double2ll_rn(td * sd * (2.0 - 3.0 * t2) / 3.0 * 0x1p62);
  row[5] = __double2ll_rn(sd * (2.0 - 15.0 * t2 + 15.0 * t2 * t2) / 15.0 * 0x1p62);
}

// tanh(y) with the table (16-byte aligned, kTanhCells rows).
__device__ __forceinline__ double tanh_tab(const long long* __restrict__ tab, double y) {
  const uint64_t bits = (uint64_t)__double_as_longlong(y);
  const uint64_t sign = bits & 0x8000000000000000ull;
  const uint64_t abits = bits ^ sign;
  if (abits < 0x3e40000000000000ull) return y;  // |y| < 2^-27, +-0, subnormals
  if (abits >= 0x4034000000000000ull) {          // |y| >= 20, +-inf, NaN
    if (abits > 0x7ff0000000000000ull) return y;
    return __longlong_as_double((long long)(sign | 0x3ff0000000000000ull));
  }
  const int e = (int)(abits >> 52) - 1023;  // -27 .. 4
  const uint64_t m = (abits & 0x000fffffffffffffull) | 0x0010000000000000ull;
  // |y| = m 2^(e - 52) = cell 2^-10 + D 2^-64
  int cell;
  uint64_t D;
  if (e >= -10) {
    const int sh = 42 - e;  // 38 .. 52
    cell = (int)(m >> sh);
    D = (m & ((1ull << sh) - 1)) << (e + 12);
  } else {
    cell = 0;
    D = e >= -12 ? m << (e + 12) : m >> (-12 - e);
  }
  const longlong2* r = reinterpret_cast<const longlong2*>(tab + kTanhRow * cell);
  const longlong2 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
  const long long d = (long long)D;  // < 2^54
  long long p = r2.y;
  p = r2.x + __mul64hi(p, d);
  p = r1.y + __mul64hi(p, d);
  p = r1.x + __mul64hi(p, d);
  p = r0.y + __mul64hi(p, d);
  const long long T = r0.x + __mul64hi(p, d);  // tanh(|y|) 2^62, in (2^35, 2^62)
  const uint64_t Tq = T >= (1ll << 62) ? (1ull << 62) - 1 : (uint64_t)T;
  return q62_to_double(Tq, sign);
}

}  // namespace wg
