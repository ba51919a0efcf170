// hilbert.cuh -- index along a Hilbert curve of a cell of a 2^10 x 2^10 x 2^10 grid (3-D)
// or of a 2^16 x 2^16 grid (2-D).
//
// J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 381 (2004): the cell
// coordinates are turned in place into the "transpose" of the Hilbert index (undo the
// excess rotations and reflections level by level, then Gray-encode), and the index is the
// bitwise interleave of the three transposed words, most significant bit of axis 0 first.
#pragma once

#include <cstdint>

namespace lpm {

// Bits 0..9 of v moved to bits 0, 3, 6, ..., 27.
__host__ __device__ inline uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__host__ __device__ inline uint32_t hilbert_index30(uint32_t x0, uint32_t x1, uint32_t x2) {
  uint32_t X[3] = {x0 & 0x3ffu, x1 & 0x3ffu, x2 & 0x3ffu};
  for (uint32_t q = 1u << 9; q > 1u; q >>= 1) {
    const uint32_t p = q - 1u;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & q) {
        X[0] ^= p;  // invert the lower bits of axis 0
      } else {
        const uint32_t t = (X[0] ^ X[i]) & p;  // exchange the lower bits of axes 0 and i
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  uint32_t t = 0;
  for (uint32_t q = 1u << 9; q > 1u; q >>= 1) {
    if (X[2] & q) t ^= q - 1u;
  }
  X[0] ^= t;
  X[1] ^= t;
  X[2] ^= t;
  return (spread10(X[0]) << 2) | (spread10(X[1]) << 1) | spread10(X[2]);
}

// Bits 0..15 of v moved to bits 0, 2, 4, ..., 30.
__host__ __device__ inline uint32_t spread16(uint32_t v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// The same construction in two dimensions, 16 bits per axis.
__host__ __device__ inline uint32_t hilbert_index2d(uint32_t x0, uint32_t x1) {
  uint32_t X[2] = {x0 & 0xffffu, x1 & 0xffffu};
  for (uint32_t q = 1u << 15; q > 1u; q >>= 1) {
    const uint32_t p = q - 1u;
    for (int i = 0; i < 2; ++i) {
      if (X[i] & q) {
        X[0] ^= p;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & p;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  uint32_t t = 0;
  for (uint32_t q = 1u << 15; q > 1u; q >>= 1) {
    if (X[1] & q) t ^= q - 1u;
  }
  X[0] ^= t;
  X[1] ^= t;
  return (spread16(X[0]) << 1) | spread16(X[1]);
}

}  // namespace lpm
