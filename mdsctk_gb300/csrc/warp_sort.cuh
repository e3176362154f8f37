// warp_sort.cuh -- sorting networks over the registers of one warp.
#pragma once
#include <cstdint>

// Ascending bitonic sort of 32 PER 64-bit keys held PER per lane (element
// e = 32 i + lane in register i): in-register compare-exchanges for the
// strides of 32 and more, shuffles below.
template <int PER>
__device__ __forceinline__ void wsort_u64(uint64_t (&v)[PER], int lane) {
#pragma unroll
  for (int k = 2; k <= 32 * PER; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int p = i ^ (j >> 5);
          if (p > i) {
            const bool up = ((i * 32 + lane) & k) == 0;
            const uint64_t a = v[i], b = v[p];
            if ((a > b) == up) {
              v[i] = b;
              v[p] = a;
            }
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < PER; ++i) {
          const int e = i * 32 + lane;
          const uint64_t o = __shfl_xor_sync(0xffffffffu, v[i], j);
          v[i] = (((e & j) == 0) == ((e & k) == 0)) ? min(v[i], o) : max(v[i], o);
        }
      }
    }
  }
}

// Element e (any e < 32 PER, per lane) of a warp-distributed array.
template <int PER>
__device__ __forceinline__ uint64_t lane_elem(const uint64_t (&v)[PER], int e) {
  uint64_t r = 0;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const uint64_t y = __shfl_sync(0xffffffffu, v[i], e & 31);
    if (i == (e >> 5)) r = y;
  }
  return r;
}


// Sums of v[i] over the 32 lanes for i < 32, the sum of v[i] returned in lane
// i (v is consumed): each step halves the values a lane holds and exchanges
// the other half with the partner lane, 31 shuffles in all instead of 32 x 5.
__device__ __forceinline__ float warp_sum_transpose32(float (&v)[32], int lane) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < o; ++i) {
      const float send = upper ? v[i] : v[i + o];
      const float keep = upper ? v[i + o] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}
