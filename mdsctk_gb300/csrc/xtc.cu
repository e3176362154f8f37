// xtc.cu -- GROMACS .xtc trajectory decoding on the GPU, feeding knn_rms
// with frames already in HBM.
//
// The reference reads trajectories through GROMACS (XTC_file,
// mdsctk.cpp:217-267; read_xtc). The format is GROMACS's published
// compressed-coordinate layout (XDR, big-endian):
//   magic 1995, natoms, step, time, box[3][3], natoms again, then either
//   3*natoms raw floats (natoms <= 9) or: precision, minint[3], maxint[3],
//   smallidx, byte count, and that many bytes (padded to 4) of a bit stream.
// The bit stream holds, atom by atom, the coordinate quantised to
// round(x * precision) - minint, packed as one mixed-radix integer of the
// three ranges (or three fixed-width fields when a range exceeds 2^24),
// followed by a flag bit; a set flag is followed by 5 bits giving the length
// of a run of atoms coded as small deltas (radix magic[smallidx]) and a
// -1/0/+1 change of smallidx. The first atom of a run is emitted before the
// large atom it follows (GROMACS swaps the first two atoms of a run, which
// makes water cheaper). Coordinates are int * (float)(1/precision).
//
// Design: the host walks the frame headers (byte counts give every frame's
// offset), the compressed bytes are copied to the device once (3-4x fewer
// bytes than the float frames), and one thread decodes one frame straight
// into the [frame][atom][xyz] float array that mds_knn_rms takes with
// MDS_DEVICE_IO. Every read is bounds-checked against the frame's end; a
// malformed frame sets an error word instead of reading past its bytes.
#include <vector>

#include "mds_common.cuh"

namespace {

// Quantisation-size table of the format (GROMACS xdrfile "magicints"):
// roughly 2^(i/3), with the format's own deviations (5060, 524287, ...).
// Decoding must use exactly these values.
__constant__ int kMagic[] = {
    0,        0,        0,        0,        0,        0,        0,        0,        0,        8,
    10,       12,       16,       20,       25,       32,       40,       50,       64,       80,
    101,      128,      161,      203,      256,      322,      406,      512,      645,      812,
    1024,     1290,     1625,     2048,     2580,     3250,     4096,     5060,     6501,     8192,
    10321,    13003,    16384,    20642,    26007,    32768,    41285,    52015,    65536,    82570,
    104031,   131072,   165140,   208063,   262144,   330280,   416127,   524287,   660561,   832255,
    1048576,  1321122,  1664510,  2097152,  2642245,  3329021,  4194304,  5284491,  6658042,  8388607,
    10568983, 13316085, 16777216};
constexpr int kFirstIdx = 9;
constexpr int kLastIdx = 72;

// XDR big-endian words
__host__ __device__ inline uint32_t be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}
__host__ __device__ inline float be_float(const unsigned char* p) {
  uint32_t u = be32(p);
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// MSB-first bit reader over [p, p + n).
struct Bits {
  const unsigned char* p;
  int64_t n, pos;
  uint32_t acc;   // last bytes read; the low `left` bits are unread
  int left;
  bool bad;
  __device__ uint32_t get(int nb) {
    uint32_t v = 0;
    while (nb >= 8) {
      if (pos >= n) { bad = true; return 0; }
      acc = (acc << 8) | p[pos++];
      v |= ((acc >> left) & 0xffu) << (nb - 8);
      nb -= 8;
    }
    if (nb > 0) {
      if (left < nb) {
        if (pos >= n) { bad = true; return 0; }
        acc = (acc << 8) | p[pos++];
        left += 8;
      }
      left -= nb;
      v |= (acc >> left) & ((1u << nb) - 1u);
    }
    return v;
  }
  // Three integers packed as one mixed-radix number of nbits bits, read as
  // little-endian bytes (the last one short); out[2], out[1] are the
  // remainders by sizes[2], sizes[1], out[0] the rest.
  __device__ void ints3(int nbits, const uint32_t sizes[3], int out[3]) {
    unsigned char by[12] = {0};
    int nb = 0;
    if (nbits > 96) { bad = true; return; }
    while (nbits > 8) {
      by[nb++] = (unsigned char)get(8);
      nbits -= 8;
    }
    if (nbits > 0) by[nb++] = (unsigned char)get(nbits);
    for (int i = 2; i > 0; --i) {
      uint32_t rem = 0;
      for (int j = nb - 1; j >= 0; --j) {
        uint32_t cur = (rem << 8) | by[j];
        uint32_t q = cur / sizes[i];
        by[j] = (unsigned char)q;
        rem = cur - q * sizes[i];
      }
      out[i] = (int)rem;
    }
    out[0] = (int)((uint32_t)by[0] | ((uint32_t)by[1] << 8) | ((uint32_t)by[2] << 16) | ((uint32_t)by[3] << 24));
  }
};

__host__ __device__ inline int bits_for(uint32_t size) {  // bits to hold 0..size-1 (xdrfile sizeofint)
  uint32_t num = 1;
  int b = 0;
  while (size >= num && b < 32) {
    ++b;
    num <<= 1;
  }
  return b;
}

// bits of the product of three ranges (xdrfile sizeofints), by byte-wise
// multiplication of the exact product
__host__ __device__ inline int bits_for3(const uint32_t s[3]) {
  uint32_t by[16] = {1};
  int nb = 1;
  for (int i = 0; i < 3; ++i) {
    uint32_t carry = 0;
    int j = 0;
    for (; j < nb; ++j) {
      carry = by[j] * s[i] + carry;
      by[j] = carry & 0xffu;
      carry >>= 8;
    }
    while (carry != 0 && j < 16) {
      by[j++] = carry & 0xffu;
      carry >>= 8;
    }
    nb = j;
  }
  int bits = 0;
  uint32_t num = 1;
  --nb;
  while (by[nb] >= num) {
    ++bits;
    num *= 2;
  }
  return bits + nb * 8;
}

// err codes written to err[frame]: 0 ok, 1 truncated, 2 natoms mismatch,
// 3 bad magic, 4 bad sizes, 5 run or smallidx out of range
__global__ void k_xtc_decode(const unsigned char* __restrict__ buf, const int64_t* __restrict__ off, int nframes,
                             int natoms, float* __restrict__ xyz, int* __restrict__ steps, float* __restrict__ times,
                             float* __restrict__ boxes, int* __restrict__ err) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nframes) return;
  const unsigned char* p = buf + off[f];
  const int64_t len = off[f + 1] - off[f];
  float* out = xyz + (int64_t)f * natoms * 3;
  int e = 0;
  if (len < 56) { err[f] = 1; return; }
  if ((int)be32(p) != 1995) { err[f] = 3; return; }
  if ((int)be32(p + 4) != natoms || (int)be32(p + 52) != natoms) { err[f] = 2; return; }
  if (steps) steps[f] = (int)be32(p + 8);
  if (times) times[f] = be_float(p + 12);
  if (boxes)
    for (int i = 0; i < 9; ++i) boxes[f * 9 + i] = be_float(p + 16 + 4 * i);
  if (natoms <= 9) {
    if (len < 56 + 12 * natoms) { err[f] = 1; return; }
    for (int i = 0; i < 3 * natoms; ++i) out[i] = be_float(p + 56 + 4 * i);
    err[f] = 0;
    return;
  }
  if (len < 56 + 36) { err[f] = 1; return; }
  const float prec = be_float(p + 56);
  int minint[3], maxint[3];
  for (int i = 0; i < 3; ++i) {
    minint[i] = (int)be32(p + 60 + 4 * i);
    maxint[i] = (int)be32(p + 72 + 4 * i);
  }
  int smallidx = (int)be32(p + 84);
  const int64_t nbytes = (int64_t)be32(p + 88);
  if (nbytes < 0 || 92 + nbytes > len || !(prec > 0.0f) || smallidx < kFirstIdx || smallidx > kLastIdx) {
    err[f] = (92 + nbytes > len) ? 1 : 4;
    return;
  }
  const float inv = (float)(1.0 / (double)prec);
  uint32_t sizeint[3], bitsizeint[3] = {0, 0, 0};
  bool large = false;
  for (int i = 0; i < 3; ++i) {
    int64_t r = (int64_t)maxint[i] - (int64_t)minint[i] + 1;
    if (r <= 0 || r > 0xffffffffll) { err[f] = 4; return; }
    sizeint[i] = (uint32_t)r;
    if (sizeint[i] > 0xffffffu) large = true;
  }
  int bitsize = 0;
  if (large)
    for (int i = 0; i < 3; ++i) bitsizeint[i] = bits_for(sizeint[i]);
  else
    bitsize = bits_for3(sizeint);
  int smaller = kMagic[smallidx - 1 > kFirstIdx ? smallidx - 1 : kFirstIdx] / 2;
  int smallnum = kMagic[smallidx] / 2;
  uint32_t sizesmall[3] = {(uint32_t)kMagic[smallidx], (uint32_t)kMagic[smallidx], (uint32_t)kMagic[smallidx]};
  Bits b{p + 92, nbytes, 0, 0u, 0, false};
  int prev[3] = {0, 0, 0};
  int run = 0, i = 0, w = 0;  // atoms consumed, atoms written
  while (i < natoms) {
    int cur[3];
    if (large) {
      for (int c = 0; c < 3; ++c) cur[c] = (int)b.get(bitsizeint[c]);
    } else {
      b.ints3(bitsize, sizeint, cur);
    }
    ++i;
    for (int c = 0; c < 3; ++c) cur[c] += minint[c];
    for (int c = 0; c < 3; ++c) prev[c] = cur[c];
    int is_smaller = 0;
    if (b.get(1)) {
      run = (int)b.get(5);
      is_smaller = run % 3;
      run -= is_smaller;
      --is_smaller;
    }
    if (b.bad) { e = 1; break; }
    if (run > 0) {
      if (i + run / 3 > natoms) { e = 5; break; }
      for (int k = 0; k < run; k += 3) {
        int t[3];
        b.ints3(smallidx, sizesmall, t);
        ++i;
        for (int c = 0; c < 3; ++c) t[c] += prev[c] - smallnum;
        if (k == 0) {
          for (int c = 0; c < 3; ++c) {
            int tmp = t[c];
            t[c] = prev[c];
            prev[c] = tmp;
          }
          for (int c = 0; c < 3; ++c) out[3 * w + c] = (float)prev[c] * inv;
          ++w;
        } else {
          for (int c = 0; c < 3; ++c) prev[c] = t[c];
        }
        for (int c = 0; c < 3; ++c) out[3 * w + c] = (float)t[c] * inv;
        ++w;
      }
    } else {
      for (int c = 0; c < 3; ++c) out[3 * w + c] = (float)cur[c] * inv;
      ++w;
    }
    if (b.bad) { e = 1; break; }
    smallidx += is_smaller;
    if (smallidx < kFirstIdx || smallidx > kLastIdx) { e = 5; break; }
    if (is_smaller < 0) {
      smallnum = smaller;
      smaller = (smallidx > kFirstIdx) ? kMagic[smallidx - 1] / 2 : 0;
    } else if (is_smaller > 0) {
      smaller = smallnum;
      smallnum = kMagic[smallidx] / 2;
    }
    sizesmall[0] = sizesmall[1] = sizesmall[2] = (uint32_t)kMagic[smallidx];
  }
  err[f] = e;
}

}  // namespace

// Walk the frame headers of an in-memory .xtc file.
extern "C" int mds_xtc_index(const unsigned char* buf, size_t len, int64_t* offsets, int max_frames, int* nframes,
                             int* natoms) {
  if (!buf || !nframes || !natoms) return MDS_ERR_ARG;
  int64_t o = 0;
  int nf = 0, na = -1;
  while (o + 56 <= (int64_t)len) {
    const unsigned char* p = buf + o;
    if ((int)be32(p) != 1995) return MDS_ERR_ARG;
    int a = (int)be32(p + 4);
    if (a < 0 || (na >= 0 && a != na)) return MDS_ERR_ARG;
    na = a;
    int64_t end;
    if (a <= 9) {
      end = o + 56 + 12 * (int64_t)a;
    } else {
      if (o + 92 > (int64_t)len) break;
      int64_t nb = (int64_t)be32(p + 88);
      end = o + 92 + ((nb + 3) / 4) * 4;
    }
    if (end > (int64_t)len) break;  // truncated last frame: dropped, as read_next_xtc stops
    if (offsets && nf < max_frames) offsets[nf] = o;
    ++nf;
    o = end;
  }
  if (offsets && nf < max_frames) offsets[nf] = o;
  *nframes = nf;
  *natoms = na < 0 ? 0 : na;
  return MDS_OK;
}

extern "C" int mds_xtc_decode(mds_ctx* ctx, const unsigned char* buf, size_t len, const int64_t* offsets,
                              int nframes, int natoms, unsigned flags, float* xyz, int* steps, float* times,
                              float* boxes) {
  if (!ctx) return MDS_ERR_ARG;
  if (!buf || !offsets || !xyz || nframes < 0 || natoms < 1) return mds_fail(ctx, MDS_ERR_ARG, "bad arguments");
  if (nframes == 0) return MDS_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const bool dev = (flags & MDS_DEVICE_IO) != 0;
  const int64_t lo = offsets[0], hi = offsets[nframes];
  if (lo < 0 || hi > (int64_t)len || hi < lo) return mds_fail(ctx, MDS_ERR_ARG, "offsets outside the buffer");
  for (int f = 0; f < nframes; ++f)
    if (offsets[f + 1] < offsets[f]) return mds_fail(ctx, MDS_ERR_ARG, "offsets not ascending");
  DevBuf db(ctx), doff(ctx), dx(ctx), derr(ctx), dst(ctx), dtm(ctx), dbx(ctx);
  MDS_TRY(db.alloc(ctx, (size_t)(hi - lo)));
  MDS_TRY(doff.alloc(ctx, sizeof(int64_t) * (nframes + 1)));
  MDS_TRY(derr.alloc(ctx, sizeof(int) * nframes));
  std::vector<int64_t> rel(nframes + 1);
  for (int f = 0; f <= nframes; ++f) rel[f] = offsets[f] - lo;
  MDS_CUDA(ctx, cudaMemcpyAsync(db.p, buf + lo, (size_t)(hi - lo), cudaMemcpyHostToDevice, s));
  MDS_CUDA(ctx, cudaMemcpyAsync(doff.p, rel.data(), sizeof(int64_t) * (nframes + 1), cudaMemcpyHostToDevice, s));
  const size_t fbytes = sizeof(float) * (size_t)nframes * natoms * 3;
  float* px = xyz;
  if (!dev) {
    MDS_TRY(dx.alloc(ctx, fbytes));
    px = dx.as<float>();
  }
  if (steps) MDS_TRY(dst.alloc(ctx, sizeof(int) * nframes));
  if (times) MDS_TRY(dtm.alloc(ctx, sizeof(float) * nframes));
  if (boxes) MDS_TRY(dbx.alloc(ctx, sizeof(float) * 9 * nframes));
  ctx->stats.launches++;
  k_xtc_decode<<<(nframes + 127) / 128, 128, 0, s>>>(db.as<unsigned char>(), doff.as<int64_t>(), nframes, natoms,
                                                     px, steps ? dst.as<int>() : nullptr,
                                                     times ? dtm.as<float>() : nullptr,
                                                     boxes ? dbx.as<float>() : nullptr, derr.as<int>());
  MDS_CUDA(ctx, cudaGetLastError());
  std::vector<int> herr(nframes);
  MDS_CUDA(ctx, cudaMemcpyAsync(herr.data(), derr.p, sizeof(int) * nframes, cudaMemcpyDeviceToHost, s));
  if (!dev) MDS_CUDA(ctx, cudaMemcpyAsync(xyz, px, fbytes, cudaMemcpyDeviceToHost, s));
  if (steps) MDS_CUDA(ctx, cudaMemcpyAsync(steps, dst.p, sizeof(int) * nframes, cudaMemcpyDeviceToHost, s));
  if (times) MDS_CUDA(ctx, cudaMemcpyAsync(times, dtm.p, sizeof(float) * nframes, cudaMemcpyDeviceToHost, s));
  if (boxes) MDS_CUDA(ctx, cudaMemcpyAsync(boxes, dbx.p, sizeof(float) * 9 * nframes, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  for (int f = 0; f < nframes; ++f)
    if (herr[f]) {
      static const char* what[] = {"", "truncated", "atom count mismatch", "bad magic", "bad sizes",
                                   "run or small-index out of range"};
      return mds_fail(ctx, MDS_ERR_ARG, "xtc frame %d: %s", f, what[herr[f] < 6 ? herr[f] : 0]);
    }
  return MDS_OK;
}
