// RANLUX "ranlxd1" stream on 48-bit integer words, usable on host and device.
//
// monofonIC's NGenIC plugin draws its white noise from GSL's gsl_rng_ranlxd1
// (src/plugins/random_ngenic.cc:44-45, 104-114).  GSL is not part of the
// reference tree; the generator is restated here from M. Luescher's published
// RANLUX algorithm (Comput. Phys. Commun. 79 (1994) 100, double-precision
// variant, luxury level 1):
//   y[n] = y[n-5] - y[n-12] - c[n-1] mod 2^48, c[n] the borrow;
//   per block 202 words are generated and the last 12 delivered in order;
//   a delivered word y maps to the uniform y * 2^-48 (exact in a double);
//   the 12 seed words come from a 31-bit shift register holding the low 31
//   seed bits: each output bit is the complement of register bit b[i], after
//   which b[i] <- b[i] xor b[i+18 mod 31] and i advances (mod 31), 48 bits per
//   word, most significant first; seed 0 means seed 1.
//
// The device keeps the 12-word history as a sliding register window so that a
// fully unrolled block uses static register indices only.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define MFX_HD __host__ __device__ __forceinline__
#else
#define MFX_HD inline
#endif

namespace mfx {

static constexpr uint64_t kMask48 = (uint64_t(1) << 48) - 1;
static constexpr double kTwoM48 = 1.0 / 281474976710656.0;  // 2^-48

struct Ranlxd1 {
  uint64_t w[12];  // y[n-12] .. y[n-1], oldest first
  uint64_t o[12];  // words of the current block still to be delivered, o[0] next
  uint32_t carry;
  int avail;

  // Seed from a value 0 <= v < 2^31 (all NGenIC column seeds are below
  // 0x7fffffff).  The 31-bit register is rotated so that bit 0 is always the
  // current tap b[i] and bit 18 the tap b[i+18].
  MFX_HD void seed31(uint32_t v) {
    if (v == 0) v = 1;
    uint32_t reg = v & 0x7fffffffu;
    // fully unrolled over the 12 words so that w[] stays in registers
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      uint64_t word = 0;
#pragma unroll 8
      for (int l = 0; l < 48; ++l) {
        const uint32_t b0 = reg & 1u;
        word = (word << 1) | uint64_t(b0 ^ 1u);
        const uint32_t nb = b0 ^ ((reg >> 18) & 1u);
        reg = (reg >> 1) | (nb << 30);
      }
      w[q] = word;
    }
    carry = 0;
    avail = 0;
  }

  MFX_HD void block() {
#pragma unroll
    for (int t = 0; t < 202; ++t) {
      uint64_t d = w[7] - w[0] - uint64_t(carry);
      carry = uint32_t(d >> 63);
      d &= kMask48;
#pragma unroll
      for (int q = 0; q < 11; ++q) w[q] = w[q + 1];
      w[11] = d;
    }
#pragma unroll
    for (int q = 0; q < 12; ++q) o[q] = w[q];
    avail = 12;
  }

  MFX_HD uint64_t next() {
    if (avail == 0) block();
    const uint64_t v = o[0];
#pragma unroll
    for (int q = 0; q < 11; ++q) o[q] = o[q + 1];
    --avail;
    return v;
  }

  MFX_HD double uniform() { return double(next()) * kTwoM48; }
};

// Host-side seeding for arbitrary `unsigned long` seeds, mirroring the 32-bit
// signed-integer arithmetic of the published seeding routine for seeds that do
// not fit in 31 bits.
inline void ranlxd1_seed_any(Ranlxd1 &r, unsigned long s) {
  if (s == 0) s = 1;
  int32_t v = int32_t(uint32_t(s & 0xffffffffUL));
  if (v >= 0) {
    r.seed31(uint32_t(v));
    return;
  }
  int bits[31];
  for (int q = 0; q < 31; ++q) { bits[q] = v % 2; v /= 2; }
  int ib = 0, jb = 18;
  for (int q = 0; q < 12; ++q) {
    // the published routine accumulates in a double; all partial values are
    // integers below 2^49 in magnitude, so int64 arithmetic is exact
    int64_t x = 0;
    for (int l = 0; l < 48; ++l) {
      x = 2 * x + int64_t((bits[ib] + 1) % 2);
      bits[ib] = (bits[ib] + bits[jb]) % 2;
      ib = (ib + 1) % 31;
      jb = (jb + 1) % 31;
    }
    r.w[q] = uint64_t(x) & kMask48;
  }
  r.carry = 0;
  r.avail = 0;
}

}  // namespace mfx
