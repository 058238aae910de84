// sm_103a kernels of the hash split.  All arithmetic is integer; values are copied as bits.
//
// Reference behaviour restated here (native-sql-engine/cpp/src/shuffle/splitter.cc):
//   hash chain + pmod + histogram          HashSplitter::ComputeAndCountPartitionId :1440-1470
//   buffer policy / emission / validity    DoSplit :855-938, AllocatePartitionBuffers :610-713,
//                                          SplitValidityBuffer :1179-1207
//   stable scatter                         DoSplit :859-874 + Split*Buffer :939-1303
#include <cuda_runtime.h>
#include <stdint.h>

#include "gz_engine.cuh"
#include "gz_kernels.h"

namespace gz {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------
// Spark Murmur3_x86_32 (hashInt / hashLong), seed chained, nulls pass the seed through.
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return __funnelshift_l(x, x, r); }
__device__ __forceinline__ uint32_t mix_k1(uint32_t k1) {
  k1 *= 0xcc9e2d51u;
  k1 = rotl32(k1, 15);
  return k1 * 0x1b873593u;
}
__device__ __forceinline__ uint32_t mix_h1(uint32_t h1, uint32_t k1) {
  h1 ^= k1;
  h1 = rotl32(h1, 13);
  return h1 * 5u + 0xe6546b64u;
}
__device__ __forceinline__ uint32_t fmix32(uint32_t h1, uint32_t len) {
  h1 ^= len;
  h1 ^= h1 >> 16;
  h1 *= 0x85ebca6bu;
  h1 ^= h1 >> 13;
  h1 *= 0xc2b2ae35u;
  h1 ^= h1 >> 16;
  return h1;
}
__device__ __forceinline__ int32_t hash_int(int32_t v, int32_t seed) {
  return (int32_t)fmix32(mix_h1((uint32_t)seed, mix_k1((uint32_t)v)), 4);
}
__device__ __forceinline__ int32_t hash_long(int64_t v, int32_t seed) {
  uint64_t u = (uint64_t)v;
  uint32_t h1 = mix_h1((uint32_t)seed, mix_k1((uint32_t)u));
  h1 = mix_h1(h1, mix_k1((uint32_t)(u >> 32)));
  return (int32_t)fmix32(h1, 8);
}
__device__ __forceinline__ int32_t pmod(int32_t h, int32_t p) {
  int32_t r = h % p;
  return r < 0 ? r + p : r;
}

__device__ __forceinline__ bool get_bit(const uint8_t* bits, uint32_t i) {
  return (bits[i >> 3] >> (i & 7)) & 1;
}
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// Clears bit `pos` of `words` for every lane with `clear`; lanes that hit the same 32-bit word
// are merged into one atomicAnd.  Must be reached by all lanes of the warp.
__device__ __forceinline__ void clear_bits(uint32_t* words, bool clear, uint32_t pos) {
  unsigned m = __ballot_sync(kFull, clear);
  if (clear) {
    uint32_t w = pos >> 5;
    unsigned peers = __match_any_sync(m, w);
    uint32_t bits = __reduce_or_sync(peers, 1u << (pos & 31));
    if ((int)lane_id() == __ffs(peers) - 1) atomicAnd(words + w, ~bits);
  }
}

// Block-wide exclusive scan of data[0..n) (u32) in place; returns the total.  Every thread
// of the block must call it.  scratch: >= 33 u32.
template <int NT>
__device__ uint32_t block_exscan(uint32_t* data, int n, uint32_t* scratch) {
  const int per = (n + NT - 1) / NT;
  const int lo = threadIdx.x * per;
  const int hi = min(lo + per, n);
  uint32_t s = 0;
  for (int i = lo; i < hi; i++) s += data[i];
  // warp inclusive scan of s
  uint32_t x = s;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if ((int)lane_id() >= o) x += y;
  }
  const int w = threadIdx.x >> 5;
  if (lane_id() == 31) scratch[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t v = (int)lane_id() < NT / 32 ? scratch[lane_id()] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, v, o);
      if ((int)lane_id() >= o) v += y;
    }
    if ((int)lane_id() < NT / 32) scratch[lane_id()] = v;
    if (lane_id() == 31) scratch[32] = v;
  }
  __syncthreads();
  uint32_t run = (w ? scratch[w - 1] : 0) + x - s;
  for (int i = lo; i < hi; i++) {
    uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
  uint32_t total = scratch[32];
  __syncthreads();
  return total;
}

// Block-wide inclusive max scan of per-thread values; returns the exclusive max for this
// thread (0 for thread 0).
template <int NT>
__device__ uint32_t block_exmax(uint32_t v, uint32_t* scratch) {
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if ((int)lane_id() >= o) x = max(x, y);
  }
  const int w = threadIdx.x >> 5;
  if (lane_id() == 31) scratch[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = (int)lane_id() < NT / 32 ? scratch[lane_id()] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, t, o);
      if ((int)lane_id() >= o) t = max(t, y);
    }
    if ((int)lane_id() < NT / 32) scratch[lane_id()] = t;
  }
  __syncthreads();
  uint32_t prev_warps = w ? scratch[w - 1] : 0;
  uint32_t xin = __shfl_up_sync(kFull, x, 1);
  uint32_t excl = lane_id() ? max(prev_warps, xin) : prev_warps;
  __syncthreads();
  return excl;
}

}  // namespace

// =======================================================================================
// k_hash_count: one CTA per tile (<= kTileRows rows of one batch).
__global__ void __launch_bounds__(256) k_hash_count(const SchemaDesc sd, const FlushDesc fd) {
  extern __shared__ uint32_t smem[];
  const TileDesc tile = fd.tiles[blockIdx.x];
  const int P = sd.P;
  const int nstr = sd.n_str;
  const ColPtr* cols = fd.cols + (size_t)tile.batch * sd.n_cols;
  uint32_t* H;
  uint32_t* BH;
  if (fd.hist_in_smem) {
    H = smem;
    BH = smem + P;
    for (int i = threadIdx.x; i < P * (1 + nstr); i += blockDim.x) smem[i] = 0;
    __syncthreads();
  } else {
    H = fd.cnt + (size_t)blockIdx.x * P;
    BH = fd.bcnt + (size_t)blockIdx.x * nstr * P;
  }

  for (uint32_t base = 0; base < tile.nrows; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const bool active = i < tile.nrows;
    const uint32_t r = tile.row0 + i;
    int32_t p = 0;
    if (active) {
      int32_t h = 42;
      for (int k = 0; k < sd.n_keys; k++) {
        const ColPtr c = cols[sd.key_col[k]];
        if (c.validity != nullptr && !get_bit(c.validity, r)) continue;
        switch (sd.key_kind[k]) {
          case KEY_I32: h = hash_int(reinterpret_cast<const int32_t*>(c.values)[r], h); break;
          case KEY_I64: h = hash_long(reinterpret_cast<const int64_t*>(c.values)[r], h); break;
          case KEY_I8: h = hash_int(reinterpret_cast<const int8_t*>(c.values)[r], h); break;
          case KEY_I16: h = hash_int(reinterpret_cast<const int16_t*>(c.values)[r], h); break;
          default: h = hash_int(get_bit(c.values, r) ? 1 : 0, h); break;
        }
      }
      p = pmod(h, P);
      fd.pids[tile.frow0 + i] = (uint16_t)p;
    }
    const unsigned amask = __ballot_sync(kFull, active);
    if (active) {
      const unsigned peers = __match_any_sync(amask, p);
      const bool leader = (int)lane_id() == __ffs(peers) - 1;
      if (leader) atomicAdd(&H[p], (uint32_t)__popc(peers));
      for (int k = 0; k < nstr; k++) {
        const ColPtr c = cols[sd.arr_col[sd.n_fixed + k]];
        const int32_t o0 = c.offsets[r], o1 = c.offsets[r + 1];
        uint32_t len = (uint32_t)(o1 - o0);
        if (o0 < 0 || o1 < o0 || (uint64_t)o1 > c.values_bytes) {
          atomicOr(fd.err, kErrBadOffsets);  // k_scatter then copies nothing
          len = 0;
        }
        const uint32_t sum = __reduce_add_sync(peers, len);
        if (leader) atomicAdd(&BH[k * P + p], sum);
      }
    }
  }

  // null counts of this tile's slice of every column (GetNullCount of the batch = sum)
  for (int a = 0; a < sd.n_array; a++) {
    const ColPtr c = cols[sd.arr_col[a]];
    if (c.validity == nullptr) continue;
    uint32_t z = 0;
    const uint32_t nbytes = (tile.nrows + 7) >> 3;
    const uint8_t* vb = c.validity + (tile.row0 >> 3);
    for (uint32_t j = threadIdx.x; j < nbytes; j += blockDim.x) {
      uint32_t byte = vb[j];
      const uint32_t rem = tile.nrows - j * 8;
      const uint32_t mask = rem >= 8 ? 0xffu : ((1u << rem) - 1);
      z += __popc(~byte & mask);
    }
    for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(kFull, z, o);
    if (lane_id() == 0 && z) atomicAdd(&fd.nullcnt[(size_t)tile.batch * sd.n_array + a], z);
  }

  if (fd.hist_in_smem) {
    __syncthreads();
    uint32_t* gh = fd.cnt + (size_t)blockIdx.x * P;
    uint32_t* gbh = fd.bcnt + (size_t)blockIdx.x * nstr * P;
    for (int i = threadIdx.x; i < P; i += blockDim.x) gh[i] = H[i];
    for (int i = threadIdx.x; i < nstr * P; i += blockDim.x) gbh[i] = BH[i];
  }
}

// =======================================================================================
// The plan: three kernels.
//   k_plan_rows  : one thread per partition walks the flush's batches in order, restating the
//                  reference's per-pid buffer policy on row counts only; writes the flush-local
//                  row / validity-bit offsets of every (tile, partition) and the emission
//                  records, and marks in rec_idx[batch][p] where a segment was cut.
//   k_plan_bytes : one thread per (binary column, partition): flush-local and in-segment byte
//                  offsets, resetting at the cuts k_plan_rows marked.
//   k_plan_scan  : exclusive scans over partitions -> output region starts.
// Counts are read ahead in groups of kAhead batches so that the serial walk is not a chain of
// dependent memory loads.
constexpr int kMaxStrPlan = 32;
constexpr int kPlanRowsThreads = 128;
constexpr int kAhead = 8;

__global__ void __launch_bounds__(kPlanRowsThreads) k_plan_rows(const SchemaDesc sd, const FlushDesc fd) {
  extern __shared__ unsigned long long psm[];
  const int NB = fd.n_batches;
  const int P = sd.P;
  const int A = sd.n_array;
  unsigned long long* hn = psm;
  unsigned long long* ihn = psm + NB;
  for (int b = threadIdx.x; b < NB; b += blockDim.x) {
    unsigned long long m = 0;
    for (int a = 0; a < A; a++)
      if (fd.nullcnt[(size_t)b * A + a]) m |= 1ull << a;
    hn[b] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // input_has_null_ is sticky and only set for the quirk columns (splitter.cc:878-886)
    unsigned long long m = *fd.st_ihn;
    for (int b = 0; b < NB; b++) {
      m |= hn[b] & sd.quirk_mask;
      ihn[b] = m;
    }
    if (blockIdx.x == 0) *fd.ihn_out = m;  // k_plan_scan stores it once everyone has read
  }
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;

  uint32_t cap = fd.st_cap[p];
  uint32_t base = fd.st_base[p];
  unsigned long long hv = fd.st_hv[p];
  uint32_t frow = 0, vpos = 0, piece_rows = 0;
  const int rec_words = kEmitFixedWords + sd.n_str;
  for (int b0 = 0; b0 < NB; b0 += kAhead) {
    uint32_t c1[kAhead];
#pragma unroll
    for (int i = 0; i < kAhead; i++) {
      const int b = b0 + i;
      c1[i] = b < NB ? fd.cnt[(size_t)fd.batches[b].tile0 * P + p] : 0u;
    }
#pragma unroll
    for (int i = 0; i < kAhead; i++) {
      const int b = b0 + i;
      if (b >= NB) break;
      const BatchDesc bd = fd.batches[b];
      uint32_t c = c1[i];
      for (uint32_t t = bd.tile0 + 1; t < bd.tile0 + bd.ntiles; t++) c += fd.cnt[(size_t)t * P + p];
      uint32_t rec = 0;
      if (c > 0) {
        const uint32_t S = bd.split_size;
        if (cap == 0 || base + c > cap) fd.call_flags[b] = 1u;
        if (cap == 0) {
          // first allocation: AllocatePartitionBuffers(max(S, cnt))
          cap = max(S, c);
          hv = ihn[b];
        } else if (base + c > cap) {
          const uint32_t ns = max(S, c);
          if (base > 0) {
            // CacheRecordBatch: the pending rows become one record batch
            const uint32_t idx = atomicAdd(fd.emit_count, 1u);
            if (idx < fd.emit_cap) {
              uint32_t* r = fd.emit + (size_t)idx * rec_words;
              r[0] = (uint32_t)p;
              r[1] = frow;
              r[2] = base;
              r[3] = (uint32_t)hv;
              r[4] = (uint32_t)(hv >> 32);
              rec = idx + 1;
            } else {
              atomicOr(fd.err, kErrEmitOverflow);
            }
            if (piece_rows) vpos = (vpos + 63u) & ~63u;
            piece_rows = 0;
            base = 0;
          }
          if (!sd.prefer_spill || ns > cap) {
            // buffers reset and reallocated: validity presence restarts from input_has_null_
            hv = ihn[b];
            cap = ns;
          }
        }
        hv |= hn[b];  // SplitValidityBuffer allocates validity for every pid with rows
        for (uint32_t t = bd.tile0; t < bd.tile0 + bd.ntiles; t++) {
          const size_t ti = (size_t)t * P + p;
          const uint32_t ct = t == bd.tile0 ? c1[i] : fd.cnt[ti];
          fd.cnt[ti] = frow;
          fd.vpos[ti] = vpos;
          frow += ct;
          vpos += ct;
          piece_rows += ct;
          base += ct;
        }
      }
      fd.rec_idx[(size_t)b * P + p] = rec;
    }
  }
  fd.st_cap[p] = cap;
  fd.st_base[p] = base;
  fd.st_hv[p] = hv;
  fd.rows_f[p] = frow;
  fd.vbits_f[p] = (vpos + 63u) & ~63u;
  fd.pstart[p] = frow;
  fd.vstart[p] = (vpos + 63u) & ~63u;
}

__global__ void __launch_bounds__(kPlanRowsThreads) k_plan_bytes(const SchemaDesc sd, const FlushDesc fd) {
  const int P = sd.P;
  const int nstr = sd.n_str;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nstr * P) return;
  const int k = idx / P, p = idx % P;
  const int T = fd.n_tiles;
  const int rec_words = kEmitFixedWords + nstr;
  uint32_t sb = fd.st_sb[(size_t)k * P + p];
  uint32_t fb = 0;
  for (int t0 = 0; t0 < T; t0 += kAhead) {
    uint32_t bc[kAhead], rec[kAhead];
#pragma unroll
    for (int i = 0; i < kAhead; i++) {
      const int t = t0 + i;
      bc[i] = 0;
      rec[i] = 0;
      if (t < T) {
        const TileDesc td = fd.tiles[t];
        bc[i] = fd.bcnt[((size_t)t * nstr + k) * P + p];
        if (td.row0 == 0) rec[i] = fd.rec_idx[(size_t)td.batch * P + p];
      }
    }
#pragma unroll
    for (int i = 0; i < kAhead; i++) {
      const int t = t0 + i;
      if (t >= T) break;
      if (rec[i]) {
        fd.emit[(size_t)(rec[i] - 1) * rec_words + kEmitFixedWords + k] = fb;
        sb = 0;
      }
      const size_t ix = ((size_t)t * nstr + k) * P + p;
      fd.bcnt[ix] = fb;
      fd.sbyte[ix] = sb;
      fb += bc[i];
      sb += bc[i];
    }
  }
  fd.st_sb[(size_t)k * P + p] = sb;
  fd.bytes_f[(size_t)k * P + p] = fb;
  fd.cstart[(size_t)k * P + p] = fb;
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_scan(const SchemaDesc sd, const FlushDesc fd) {
  __shared__ uint32_t scan_scratch[33];
  const int P = sd.P;
  block_exscan<kPlanThreads>(fd.pstart, P, scan_scratch);
  block_exscan<kPlanThreads>(fd.vstart, P, scan_scratch);
  for (int k = 0; k < sd.n_str; k++) block_exscan<kPlanThreads>(fd.cstart + (size_t)k * P, P, scan_scratch);
  if (threadIdx.x == 0) *fd.st_ihn = *fd.ihn_out;
}

// =======================================================================================
// k_scatter: one CTA per tile.
namespace {
constexpr int kW = kScatterThreads / 32;

// One stable LSD pass over 8 bits of the keys.
__device__ void radix_pass(const uint16_t* kin, const uint16_t* pin, uint16_t* kout,
                           uint16_t* pout, int n, int shift, uint16_t* wcnt, uint32_t* off,
                           uint32_t* scratch) {
  const int w = threadIdx.x >> 5;
  const int seg = ((n + kW * 32 - 1) / (kW * 32)) * 32;
  for (int i = threadIdx.x; i < kW * 256; i += blockDim.x) wcnt[i] = 0;
  __syncthreads();
  for (int c = 0; c < seg; c += 32) {
    const int i = w * seg + c + lane_id();
    const bool act = i < n;
    const unsigned m = __ballot_sync(kFull, act);
    if (act) {
      const unsigned d = (kin[i] >> shift) & 255u;
      const unsigned peers = __match_any_sync(m, d);
      if ((int)lane_id() == __ffs(peers) - 1) wcnt[w * 256 + d] += (uint16_t)__popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kW * 256; i += blockDim.x) {
    const int d = i / kW, ww = i % kW;
    off[i] = wcnt[ww * 256 + d];
  }
  __syncthreads();
  block_exscan<kScatterThreads>(off, kW * 256, scratch);
  for (int c = 0; c < seg; c += 32) {
    const int i = w * seg + c + lane_id();
    const bool act = i < n;
    const unsigned m = __ballot_sync(kFull, act);
    unsigned d = 0, peers = 0;
    if (act) {
      d = (kin[i] >> shift) & 255u;
      peers = __match_any_sync(m, d);
      const unsigned rank = __popc(peers & ((1u << lane_id()) - 1));
      const uint32_t pos = off[d * kW + w] + rank;
      kout[pos] = kin[i];
      pout[pos] = pin[i];
    }
    __syncwarp();
    if (act && (int)lane_id() == __ffs(peers) - 1) off[d * kW + w] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ void copy_rows(uint8_t* out, const uint8_t* in, const uint16_t* ps,
                                          const uint32_t* dstrow, uint32_t row0, int n) {
  T* o = reinterpret_cast<T*>(out);
  const T* s = reinterpret_cast<const T*>(in) + row0;
  for (int j = threadIdx.x; j < n; j += blockDim.x) o[dstrow[j]] = s[ps[j]];
}
}  // namespace

__global__ void __launch_bounds__(kScatterThreads) k_scatter(const SchemaDesc sd, const FlushDesc fd) {
  extern __shared__ __align__(16) uint8_t ssm[];
  __shared__ uint32_t scratch[33];
  const int T = kTileRows;
  uint16_t* kA = reinterpret_cast<uint16_t*>(ssm);          // [T]
  uint16_t* pA = kA + T;                                    // [T]
  uint16_t* kB = pA + T;                                    // [T]
  uint16_t* pB = kB + T;                                    // [T]
  uint32_t* dbit = reinterpret_cast<uint32_t*>(pB + T);     // [T] (radix offsets while sorting)
  uint16_t* rs = reinterpret_cast<uint16_t*>(dbit + T);     // [T]
  uint32_t* S = reinterpret_cast<uint32_t*>(rs + T);        // [T + 1]
  uint16_t* wcnt = reinterpret_cast<uint16_t*>(S + T + 1);  // [kW * 256]

  const TileDesc tile = fd.tiles[blockIdx.x];
  const int n = (int)tile.nrows;
  const int P = sd.P;
  const int nstr = sd.n_str;
  const ColPtr* cols = fd.cols + (size_t)tile.batch * sd.n_cols;
  if (*reinterpret_cast<volatile int32_t*>(fd.err) != 0) return;  // inputs rejected by k_hash_count

  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    kA[j] = fd.pids[tile.frow0 + j];
    pA[j] = (uint16_t)j;
  }
  __syncthreads();
  radix_pass(kA, pA, kB, pB, n, 0, wcnt, dbit, scratch);
  uint16_t* ks = kB;
  uint16_t* ps = pB;
  uint32_t* dstrow = reinterpret_cast<uint32_t*>(kA);  // kA,pA are free after one pass
  if (P > 256) {
    radix_pass(kB, pB, kA, pA, n, 8, wcnt, dbit, scratch);
    ks = kA;
    ps = pA;
    dstrow = reinterpret_cast<uint32_t*>(kB);
  }

  // run starts: rs[j] = first sorted position with the same partition id
  {
    const int per = (n + kScatterThreads - 1) / kScatterThreads;
    const int lo = threadIdx.x * per;
    const int hi = min(lo + per, n);
    uint32_t mx = 0;
    for (int j = lo; j < hi; j++)
      if (j == 0 || ks[j] != ks[j - 1]) mx = j;
    uint32_t carry = block_exmax<kScatterThreads>(mx, scratch);
    for (int j = lo; j < hi; j++) {
      if (j == 0 || ks[j] != ks[j - 1]) carry = j;
      rs[j] = (uint16_t)carry;
    }
  }
  __syncthreads();
  const size_t tp = (size_t)blockIdx.x * P;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int p = ks[j];
    const uint32_t rk = (uint32_t)(j - rs[j]);
    dstrow[j] = fd.pstart[p] + fd.cnt[tp + p] + rk;
    dbit[j] = fd.vstart[p] + fd.vpos[tp + p] + rk;
  }
  __syncthreads();

  const uint32_t row0 = tile.row0;
  for (int a = 0; a < sd.n_array; a++) {
    const ColPtr c = cols[sd.arr_col[a]];
    const int kind = sd.arr_kind[a];
    // validity: clear the bits of null rows (destination words start 0xff)
    if (c.validity != nullptr && fd.out_valid[a] != nullptr &&
        fd.nullcnt[(size_t)tile.batch * sd.n_array + a] != 0) {
      uint32_t* ow = fd.out_valid[a];
      for (int j0 = 0; j0 < n; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        bool clr = false;
        uint32_t pos = 0;
        if (j < n) {
          clr = !get_bit(c.validity, row0 + ps[j]);
          pos = dbit[j];
        }
        clear_bits(ow, clr, pos);
      }
    }
    if (kind == COL_FIXED) {
      switch (sd.arr_width[a]) {
        case 1: copy_rows<uint8_t>(fd.out_values[a], c.values, ps, dstrow, row0, n); break;
        case 2: copy_rows<uint16_t>(fd.out_values[a], c.values, ps, dstrow, row0, n); break;
        case 4: copy_rows<uint32_t>(fd.out_values[a], c.values, ps, dstrow, row0, n); break;
        case 8: copy_rows<uint64_t>(fd.out_values[a], c.values, ps, dstrow, row0, n); break;
        default: copy_rows<uint4>(fd.out_values[a], c.values, ps, dstrow, row0, n); break;
      }
    } else if (kind == COL_BOOL) {
      uint32_t* ow = fd.out_bits[a];
      for (int j0 = 0; j0 < n; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        bool clr = false;
        uint32_t pos = 0;
        if (j < n) {
          clr = !get_bit(c.values, row0 + ps[j]);
          pos = dbit[j];
        }
        clear_bits(ow, clr, pos);
      }
    } else {
      const int k = sd.arr_str[a];
      const int32_t* oin = c.offsets + row0;
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const int r = ps[j];
        S[j] = (uint32_t)(oin[r + 1] - oin[r]);
      }
      __syncthreads();
      const uint32_t total = block_exscan<kScatterThreads>(S, n, scratch);
      if (threadIdx.x == 0) S[n] = total;
      __syncthreads();
      int32_t* ooff = reinterpret_cast<int32_t*>(fd.out_values[a]);
      const size_t tk = ((size_t)blockIdx.x * nstr + k) * P;
      const uint32_t* cst = fd.cstart + (size_t)k * P;
      uint8_t* ochars = fd.out_chars[a];
      // offsets, one row per thread; then characters, one string per warp step
      for (int j0 = 0; j0 < n; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        const uint8_t* src = nullptr;
        uint8_t* dst = nullptr;
        uint32_t len = 0;
        if (j < n) {
          const int p = ks[j];
          const uint32_t pref = S[j] - S[rs[j]];
          len = S[j + 1] - S[j];
          ooff[dstrow[j]] = (int32_t)(fd.sbyte[tk + p] + pref + len);
          src = c.values + oin[ps[j]];
          dst = ochars + cst[p] + fd.bcnt[tk + p] + pref;
        }
        for (int s = 0; s < 32; s++) {
          const uint8_t* ss = reinterpret_cast<const uint8_t*>(
              __shfl_sync(kFull, reinterpret_cast<unsigned long long>(src), s));
          uint8_t* dd = reinterpret_cast<uint8_t*>(
              __shfl_sync(kFull, reinterpret_cast<unsigned long long>(dst), s));
          const uint32_t ll = __shfl_sync(kFull, len, s);
          for (uint32_t x = lane_id(); x < ll; x += 32) dd[x] = ss[x];
        }
      }
      __syncthreads();
    }
  }
}

// =======================================================================================
// launch helpers
cudaError_t launch_hash_count(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  const size_t sm = fd.hist_in_smem ? sizeof(uint32_t) * sd.P * (1 + sd.n_str) : 0;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_hash_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  k_hash_count<<<fd.n_tiles, 256, sm, st>>>(sd, fd);
  return cudaGetLastError();
}

cudaError_t launch_plan(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  const size_t sm = sizeof(unsigned long long) * 2 * fd.n_batches;
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_plan_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  k_plan_rows<<<(sd.P + kPlanRowsThreads - 1) / kPlanRowsThreads, kPlanRowsThreads, sm, st>>>(sd, fd);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (sd.n_str > 0) {
    const int n = sd.n_str * sd.P;
    k_plan_bytes<<<(n + kPlanRowsThreads - 1) / kPlanRowsThreads, kPlanRowsThreads, 0, st>>>(sd, fd);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_plan_scan<<<1, kPlanThreads, 0, st>>>(sd, fd);
  return cudaGetLastError();
}

size_t scatter_smem_bytes() {
  const int T = kTileRows;
  return 4 * sizeof(uint16_t) * T + sizeof(uint32_t) * T + sizeof(uint16_t) * T +
         sizeof(uint32_t) * (T + 1) + sizeof(uint16_t) * kW * 256;
}

cudaError_t launch_scatter(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  const size_t sm = scatter_smem_bytes();
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  k_scatter<<<fd.n_tiles, kScatterThreads, sm, st>>>(sd, fd);
  return cudaGetLastError();
}

int max_str_columns() { return kMaxStrPlan; }

}  // namespace gz
