// tc_select.cuh -- warp radix selection of the best K' keys of a candidate
// list (the compaction step of the tensor-core screens).
#pragma once

#include "knn_common.cuh"

#define TC_CAPG 512  // keys per (row, column segment) list
// Radix search over the keys held in registers (PER per lane, invalid keys
// = MDS_KEY_INF): starting from the digits (mask, prefix) that every valid
// key shares, refine (mask, prefix) byte by byte until the keys whose
// processed digits are <= prefix's are exactly the `need` smallest (the
// search stops as soon as the digit bucket holding the need-th key is whole).
template <int PER>
__device__ inline void warp_radix_find(const uint64_t (&kv)[PER], int start_pass, uint64_t& mask, uint64_t& prefix,
                                       int need, int* hist, int lane) {
  for (int pass = start_pass; pass >= 0; --pass) {
    const int sh = pass * 8;
    for (int b = lane; b < 256; b += 32) hist[b] = 0;
    __syncwarp();
#pragma unroll
    for (int i = 0; i < PER; ++i)
      if (kv[i] != MDS_KEY_INF && (kv[i] & mask) == prefix) atomicAdd(&hist[(int)((kv[i] >> sh) & 255u)], 1);
    __syncwarp();
    int c[8], loc = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      c[b] = hist[8 * lane + b];
      loc += c[b];
    }
    int inc = loc;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const int exc = inc - loc;
    int digit = -1, before = 0, cnt = 0;
    if (exc < need && need <= inc) {
      int acc = exc;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        if (digit < 0 && acc + c[b] >= need) {
          digit = 8 * lane + b;
          before = acc;
          cnt = c[b];
        }
        acc += c[b];
      }
    }
    const unsigned own = __ballot_sync(0xffffffffu, digit >= 0);
    const int src_lane = __ffs(own) - 1;
    digit = __shfl_sync(0xffffffffu, digit, src_lane);
    before = __shfl_sync(0xffffffffu, before, src_lane);
    cnt = __shfl_sync(0xffffffffu, cnt, src_lane);
    __syncwarp();
    need -= before;
    prefix |= (uint64_t)digit << sh;
    mask |= (uint64_t)255 << sh;
    if (cnt == need) break;  // the whole bucket is kept
  }
}

// Keep the Kp smallest of the keys src[0, n0) and src[off1, off1 + n1) (at
// most TC_CAPG slots in all: off1 + n1 <= TC_CAPG) in src[0..Kp), unsorted,
// and return the largest kept value: a most-significant-digit radix select
// over the 64-bit keys (8-bit digits, stopping as soon as the digit bucket
// holding the Kp-th key is kept whole), then a ballot compaction. hist: 256
// ints of this warp's shared scratch. With rank2 (1 <= rank2 <= Kp, and at
// least rank2 keys present), *v2 receives the value of the rank2-th smallest
// key, found by a second search over the same registers; with Kp = 0 only
// that value is found (the list is left as it is, the return value is +inf).
__device__ inline float warp_select_keep2(uint64_t* src, int n0, int off1, int n1, int Kp, int* hist, int lane,
                                          int rank2 = 0, float* v2 = nullptr) {
  constexpr int PER = TC_CAPG / 32;
  uint64_t kv[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int x = lane + 32 * i;
    kv[i] = (x < n0 || (x >= off1 && x < off1 + n1)) ? src[x] : MDS_KEY_INF;
  }
  // Leading bytes that every valid key shares (values of one magnitude share
  // their sign/exponent byte) are skipped: their histogram would put all keys
  // in one bucket, one shared-memory atomic after another.
  uint32_t hmin = 0xffffffffu, hmax = 0u;
#pragma unroll
  for (int i = 0; i < PER; ++i)
    if (kv[i] != MDS_KEY_INF) {
      const uint32_t hv = (uint32_t)(kv[i] >> 32);
      hmin = min(hmin, hv);
      hmax = max(hmax, hv);
    }
  hmin = __reduce_min_sync(0xffffffffu, hmin);
  hmax = __reduce_max_sync(0xffffffffu, hmax);
  const int same_bytes = (hmin <= hmax) ? ((hmin == hmax) ? 4 : __clz(hmin ^ hmax) / 8) : 0;
  const uint64_t mask0 = same_bytes ? (~0ull << (64 - 8 * same_bytes)) : 0ull;
  const uint64_t prefix0 = ((uint64_t)hmin << 32) & mask0;
  if (rank2 > 0) {
    uint64_t mask = mask0, prefix = prefix0;
    warp_radix_find(kv, 7 - same_bytes, mask, prefix, rank2, hist, lane);
    float vm = 0.0f;
#pragma unroll
    for (int i = 0; i < PER; ++i)
      if (kv[i] != MDS_KEY_INF && (kv[i] & mask) <= prefix) vm = fmaxf(vm, mds_key_value(kv[i]));
    for (int o = 16; o > 0; o >>= 1) vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    *v2 = vm;
  }
  if (Kp <= 0) {  // the rank2 value only: nothing kept or moved
    __syncwarp();
    return INFINITY;
  }
  uint64_t mask = mask0, prefix = prefix0;
  warp_radix_find(kv, 7 - same_bytes, mask, prefix, Kp, hist, lane);
  // keep every key whose processed digits are <= prefix's
  int base = 0;
  float vmax = 0.0f;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const bool keep = kv[i] != MDS_KEY_INF && (kv[i] & mask) <= prefix;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      src[base + __popc(bal & ((1u << lane) - 1u))] = kv[i];
      vmax = fmaxf(vmax, mds_key_value(kv[i]));
    }
    base += __popc(bal);
  }
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  __syncwarp();
  return vmax;
}

// One contiguous list src[0, n), n <= TC_CAPG.
__device__ inline float warp_select_keep(uint64_t* src, int n, int Kp, int* hist, int lane) {
  return warp_select_keep2(src, n, TC_CAPG, 0, Kp, hist, lane);
}
