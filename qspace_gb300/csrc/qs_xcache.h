// Device-resident table of CG / X-symbol factors (qs_xcache_*): the view the
// kernels read, the probe rule shared by the host mirror and the device, and
// the per-call factor source of the keyed grouped GEMM.
//
// The reference keeps X-symbols in a host hash map (X3Map gXS,
// Source/clebsch.hh:3911-4245) filled by X3Map::contractCGR
// (Source/clebsch_aux.cc:4073-4330) and consulted once per block pair inside
// the pair loop.  Here a caller derives a 128-bit key from the same
// (CGT_a, ica, CGT_b, icb) tuple, puts the factors once, and the products
// resolve them on the device.
#pragma once

#include <cstdint>

#include "qs_internal.h"

namespace qs {

// Open addressing with linear probing over a power-of-two capacity; an empty
// slot holds the reserved key (2^64-1, 2^64-1).  The table is at most 3/4
// full, so every probe sequence reaches an empty slot.
constexpr uint64_t XKEY_EMPTY = ~0ull;

struct XView {
  const uint64_t *keys;  // 2 words per slot
  const double *vals;
  uint64_t mask;         // capacity - 1
};

// Slot hash of a key (splitmix64-style finaliser over both words).
__host__ __device__ inline uint64_t xkey_hash(uint64_t a, uint64_t b) {
  uint64_t h = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull;
  h ^= h >> 31;
  h *= 0x94D049BB133111EBull;
  h ^= h >> 29;
  return h;
}

__device__ inline bool xview_find(const XView &v, uint64_t a, uint64_t b, double *out) {
  uint64_t i = xkey_hash(a, b) & v.mask;
  for (uint64_t n = 0; n <= v.mask; ++n, i = (i + 1) & v.mask) {
    const uint64_t ka = v.keys[2 * i], kb = v.keys[2 * i + 1];
    if (ka == a && kb == b) {
      *out = v.vals[i];
      return true;
    }
    if (ka == XKEY_EMPTY && kb == XKEY_EMPTY) return false;
  }
  return false;
}

// qs_xcache.cu: frees the device memory of every table of a context that is
// being destroyed; the tables stay valid handles (unusable, destroyable)
void xcache_orphan_all(Ctx *ctx);

}  // namespace qs
