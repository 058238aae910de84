// sm_103a kernels of the hash split.  All arithmetic is integer; values are copied as bits.
//
// Reference behaviour restated here (native-sql-engine/cpp/src/shuffle/splitter.cc):
//   hash chain + pmod + histogram          HashSplitter::ComputeAndCountPartitionId :1440-1470
//   round-robin / range partition ids      RoundRobinSplitter :1379-1387, FallbackRangeSplitter :1499-1519
//   buffer policy / emission / validity    DoSplit :855-938, AllocatePartitionBuffers :610-713,
//                                          SplitValidityBuffer :1179-1207
//   stable scatter                         DoSplit :859-874 + Split*Buffer :939-1303
#include <cuda_runtime.h>
#include <stdint.h>

#include "gz_engine.cuh"
#include "gz_hash.cuh"
#include "gz_kernels.h"

namespace gz {

namespace {

using namespace hash;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// Barrier over the NT threads 0..NT-1: the whole block (BAR 0) or named barrier BAR.
template <int NT, int BAR>
__device__ __forceinline__ void group_sync() {
  if constexpr (BAR == 0) __syncthreads();
  else asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NT) : "memory");
}

// Exclusive scan of data[0..n) (u32) in place over threads 0..NT-1; returns the total.  Every
// one of them must call it.  scratch: >= 33 u32.
template <int NT, int BAR = 0>
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
  group_sync<NT, BAR>();
  if (w == 0) {
    uint32_t v = (int)lane_id() < NT / 32 ? scratch[lane_id()] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, v, o);
      if ((int)lane_id() >= o) v += y;
    }
    if ((int)lane_id() < NT / 32) scratch[lane_id()] = v;
    if (lane_id() == 31) scratch[32] = v;
  }
  group_sync<NT, BAR>();
  uint32_t run = (w ? scratch[w - 1] : 0) + x - s;
  for (int i = lo; i < hi; i++) {
    uint32_t v = data[i];
    data[i] = run;
    run += v;
  }
  uint32_t total = scratch[32];
  group_sync<NT, BAR>();
  return total;
}

// Inclusive max scan of per-thread values over threads 0..NT-1; returns the exclusive max for
// this thread (0 for thread 0).
template <int NT, int BAR = 0>
__device__ uint32_t block_exmax(uint32_t v, uint32_t* scratch) {
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if ((int)lane_id() >= o) x = max(x, y);
  }
  const int w = threadIdx.x >> 5;
  if (lane_id() == 31) scratch[w] = x;
  group_sync<NT, BAR>();
  if (w == 0) {
    uint32_t t = (int)lane_id() < NT / 32 ? scratch[lane_id()] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, t, o);
      if ((int)lane_id() >= o) t = max(t, y);
    }
    if ((int)lane_id() < NT / 32) scratch[lane_id()] = t;
  }
  group_sync<NT, BAR>();
  uint32_t prev_warps = w ? scratch[w - 1] : 0;
  uint32_t xin = __shfl_up_sync(kFull, x, 1);
  uint32_t excl = lane_id() ? max(prev_warps, xin) : prev_warps;
  group_sync<NT, BAR>();
  return excl;
}

}  // namespace

// =======================================================================================
// k_hash_count: one CTA per segment (<= seg_tiles * kTileRows rows of one batch).
constexpr int kMaxStrPlan = kMaxCols;  // binary, list and nested-stream columns

constexpr int kHashThreads = 256;
constexpr int kHashRows = kTileRows / kHashThreads;  // rows of a tile per thread
static_assert(kHashRows * kHashThreads == kTileRows, "hash rows per thread");

// kLists: the schema has list columns (instantiated apart so the other schemas' code is unchanged)
template <bool kLists>
__global__ void __launch_bounds__(kHashThreads) k_hash_count(const SchemaDesc sd, const FlushDesc fd) {
  extern __shared__ uint32_t smem[];
  __shared__ ColPtr s_key[kMaxKeys];
  __shared__ int32_t s_kind[kMaxKeys];
  __shared__ ColPtr s_str[kMaxStrPlan];
  const SegDesc tile = fd.segs[blockIdx.x];
  const int P = sd.P;
  const int nstr = sd.n_str;
  const int nkeys = sd.n_keys;
  const ColPtr* cols = fd.cols + (size_t)tile.batch * sd.n_cols;
  if (threadIdx.x < nkeys) {
    s_key[threadIdx.x] = cols[sd.key_col[threadIdx.x]];
    s_kind[threadIdx.x] = sd.key_kind[threadIdx.x];
  }
  if (threadIdx.x < nstr) s_str[threadIdx.x] = cols[sd.arr_col[sd.n_fixed + threadIdx.x]];
  uint32_t* H;
  uint32_t* BH;
  if (fd.hist_in_smem) {
    H = smem;
    BH = smem + P;
    for (int i = threadIdx.x; i < P * (1 + nstr); i += blockDim.x) smem[i] = 0;
  } else {
    H = fd.cnt + (size_t)blockIdx.x * P;
    BH = fd.bcnt + (size_t)blockIdx.x * nstr * P;
  }
  __syncthreads();
  const unsigned long long M = sd.pmod_magic;
  const int part = sd.partitioner;
  bool bad = false;
  bool bad_pid = false;
  // tile by tile; before every tile after the first, the counts so far are the tile's prefix
  for (uint32_t t0 = 0; t0 < tile.nrows; t0 += kTileRows) {
  if (t0 > 0 && fd.tilepre != nullptr) {
    __syncthreads();  // every row of the earlier tiles is counted
    const size_t ti = (size_t)tile.tile0 + t0 / kTileRows;
    for (int q = threadIdx.x; q < P; q += blockDim.x) fd.tilepre[ti * P + q] = H[q];
    for (int q = threadIdx.x; q < nstr * P; q += blockDim.x) fd.tilebpre[ti * nstr * P + q] = BH[q];
    __syncthreads();  // the copies are read before the next tile's rows are added
  }
  const uint32_t t1 = min(tile.nrows, t0 + (uint32_t)kTileRows);
  // rows i0 .. i0 + 3 (i0 = t0 + 4 * thread) of the tile: a whole group is loaded with 16-byte
  // vector loads when the column's buffer is 16-byte aligned (the group's first row is a
  // multiple of 4, so then every group is), otherwise and for the tile's last partial group row
  // by row; all loads of a column are issued before any is used
  const uint32_t i0 = t0 + kHashRows * threadIdx.x;
  const uint32_t m = i0 < t1 ? min((uint32_t)kHashRows, t1 - i0) : 0u;  // rows of this thread
  const uint32_t r0 = tile.row0 + (m ? i0 : t1 - 1);  // a thread without rows reads a valid one
  const bool whole = m == kHashRows;
  bool act[kHashRows];
  uint32_t rr[kHashRows];
  int32_t h[kHashRows];
#pragma unroll
  for (int u = 0; u < kHashRows; u++) {
    act[u] = u < m;
    rr[u] = act[u] ? r0 + u : r0;
    h[u] = 42;
  }
  for (int k = 0; k < nkeys; k++) {
    const ColPtr c = s_key[k];
    const int kind = s_kind[k];
    int64_t v[kHashRows];
    bool valid[kHashRows];
    const bool aligned16 = (reinterpret_cast<uintptr_t>(c.values) & 15) == 0;
    if (whole && aligned16 && kind == KEY_I64) {
      const longlong2 a0 = reinterpret_cast<const longlong2*>(c.values)[r0 >> 1];
      const longlong2 a1 = reinterpret_cast<const longlong2*>(c.values)[(r0 >> 1) + 1];
      v[0] = a0.x;
      v[1] = a0.y;
      v[2] = a1.x;
      v[3] = a1.y;
    } else if (whole && aligned16 && kind == KEY_I32) {
      const int4 a0 = reinterpret_cast<const int4*>(c.values)[r0 >> 2];
      v[0] = a0.x;
      v[1] = a0.y;
      v[2] = a0.z;
      v[3] = a0.w;
    } else if (kind == KEY_STR) {
#pragma unroll
      for (int u = 0; u < kHashRows; u++) v[u] = 0;  // hashed below from the offsets
    } else {
#pragma unroll
      for (int u = 0; u < kHashRows; u++) {
        const uint32_t r = rr[u];
        switch (kind) {
          case KEY_I32: v[u] = reinterpret_cast<const int32_t*>(c.values)[r]; break;
          case KEY_I64: v[u] = reinterpret_cast<const int64_t*>(c.values)[r]; break;
          case KEY_I8: v[u] = reinterpret_cast<const int8_t*>(c.values)[r]; break;
          case KEY_I16: v[u] = reinterpret_cast<const int16_t*>(c.values)[r]; break;
          default: v[u] = get_bit(c.values, r) ? 1 : 0; break;
        }
      }
    }
    if (part == PART_RANGE) {  // the values are the partition ids; their validity is not read
#pragma unroll
      for (int u = 0; u < kHashRows; u++) h[u] = (int32_t)v[u];
      continue;
    }
#pragma unroll
    for (int u = 0; u < kHashRows; u++) valid[u] = c.validity == nullptr || get_bit(c.validity, rr[u]);
    if (kind == KEY_STR) {
      // utf8 key: offsets were checked against the characters by Split (host inputs) or are the
      // caller's device buffers
#pragma unroll
      for (int u = 0; u < kHashRows; u++) {
        if (!valid[u] || !act[u]) continue;
        const int32_t o0 = c.offsets[rr[u]], o1 = c.offsets[rr[u] + 1];
        if (o0 < 0 || o1 < o0 || (uint64_t)o1 > c.values_bytes) {
          bad = true;
          continue;
        }
        h[u] = hash_bytes(c.values + o0, o1 - o0, h[u]);
      }
      continue;
    }
#pragma unroll
    for (int u = 0; u < kHashRows; u++)  // null: seed passes
      if (valid[u]) h[u] = kind == KEY_I64 ? hash_long(v[u], h[u]) : hash_int((int32_t)v[u], h[u]);
  }
  uint32_t p[kHashRows];
#pragma unroll
  for (int u = 0; u < kHashRows; u++) {
    if (part == PART_HASH) {
      p[u] = fast_pmod(h[u], (uint32_t)P, M);
    } else if (part == PART_RR) {
      // the selection runs on from row to row and batch to batch, wrapping at P
      p[u] = fastmod_u32(fd.rr_base + tile.frow0 + i0 + u, (uint32_t)P, M);
    } else {
      p[u] = (uint32_t)h[u];
      if (p[u] >= (uint32_t)P) {  // negative or too large: the batch is rejected
        bad_pid |= act[u];
        p[u] = 0;
      }
    }
    if (act[u]) fd.pids[tile.frow0 + i0 + u] = (uint16_t)p[u];
    if (part == PART_RR) {  // consecutive rows, distinct partitions: nothing to aggregate
      if (act[u]) atomicAdd(&H[p[u]], 1u);
    } else {
      // warp-aggregated: the lanes whose row went to the same partition add once (skewed keys
      // otherwise serialise on one counter)
      const unsigned grp = __match_any_sync(kFull, act[u] ? p[u] : 0xffffffffu);
      if (act[u] && (int)lane_id() == __ffs(grp) - 1) atomicAdd(&H[p[u]], (uint32_t)__popc(grp));
    }
  }
  for (int k = 0; k < nstr; k++) {
    const ColPtr c = s_str[k];
    // o[u] = offsets[r0 + min(u, m)]: row u < m spans o[u] .. o[u + 1]; 64-bit offsets of
    // large binary columns are read as such and checked like the 32-bit ones
    int64_t o[kHashRows + 1];
    const bool aligned = (reinterpret_cast<uintptr_t>(c.offsets) & 15) == 0;
    if (sd.arr_width[sd.n_fixed + k] == 8) {
      const int64_t* o64 = reinterpret_cast<const int64_t*>(c.offsets);
      if (whole && aligned) {
        const longlong2 a0 = reinterpret_cast<const longlong2*>(o64)[r0 >> 1];
        const longlong2 a1 = reinterpret_cast<const longlong2*>(o64)[(r0 >> 1) + 1];
        o[0] = a0.x;
        o[1] = a0.y;
        o[2] = a1.x;
        o[3] = a1.y;
        o[4] = o64[r0 + kHashRows];
      } else {
#pragma unroll
        for (int u = 0; u <= kHashRows; u++) o[u] = o64[r0 + min((uint32_t)u, m)];
      }
    } else if (whole && aligned) {
      const int4 a0 = reinterpret_cast<const int4*>(c.offsets)[r0 >> 2];
      o[0] = a0.x;
      o[1] = a0.y;
      o[2] = a0.z;
      o[3] = a0.w;
      o[4] = c.offsets[r0 + kHashRows];
    } else {
#pragma unroll
      for (int u = 0; u <= kHashRows; u++) o[u] = c.offsets[r0 + min((uint32_t)u, m)];
    }
    // a list column: element offsets, elements of 1 << shift bytes, a null row has none
    const int ak = sd.n_fixed + k;
    const int shift = kLists ? sd.arr_shift[ak] : 0;
    const bool list = kLists && ((sd.list_mask >> ak) & 1ull);
    // readable elements: bytes, or bits of a list of bool elements
    const uint64_t cap = kLists && ((sd.listbit_mask >> ak) & 1ull) ? c.values_bytes * 8 : c.values_bytes;
#pragma unroll
    for (int u = 0; u < kHashRows; u++) {
      uint32_t len = (uint32_t)(o[u + 1] - o[u]) << shift;
      if (act[u] && (o[u] < 0 || o[u + 1] < o[u] || ((uint64_t)o[u + 1] << shift) > cap)) {
        bad = true;
        len = 0;
      }
      if (list && c.validity != nullptr && !get_bit(c.validity, rr[u])) len = 0;
      if (act[u] && len) atomicAdd(&BH[k * P + p[u]], len);
    }
  }
  // offsets of the tile's first and one-past-last row (k_scatter stages the characters between)
  if (threadIdx.x < nstr) {
    const ColPtr c = s_str[threadIdx.x];
    const size_t ct = ((size_t)tile.tile0 + t0 / kTileRows) * nstr + threadIdx.x;
    // (valid offsets of either width are below 2^31: a batch's characters are at most that)
    const int sh = kLists ? sd.arr_shift[sd.n_fixed + threadIdx.x] : 0;  // list: element bytes
    if (sd.arr_width[sd.n_fixed + threadIdx.x] == 8) {
      const int64_t* o64 = reinterpret_cast<const int64_t*>(c.offsets);
      fd.crange[ct] = make_int2((int32_t)o64[tile.row0 + t0], (int32_t)o64[tile.row0 + t1]);
    } else {
      fd.crange[ct] = make_int2(c.offsets[tile.row0 + t0] << sh, c.offsets[tile.row0 + t1] << sh);
    }
  }
  }
  if (bad) atomicOr(fd.err, kErrBadOffsets);  // k_scatter then copies nothing
  if (bad_pid) atomicOr(fd.err, kErrBadPid);

  // null counts of this segment's slice of every column (GetNullCount of the batch = sum): one
  // warp per column, 32 rows per 4-byte word when the slice is word aligned, else byte by byte
  {
    const int lane = (int)lane_id();
    const int nwarps = (int)(blockDim.x >> 5);
    const uint32_t nbytes = (tile.nrows + 7) >> 3;
    for (int a = (int)(threadIdx.x >> 5); a < sd.n_array; a += nwarps) {
      const uint8_t* validity = cols[sd.arr_col[a]].validity;
      if (validity == nullptr) continue;
      const uint8_t* vb = validity + (tile.row0 >> 3);
      uint32_t z = 0;
      uint32_t j0 = 0;  // first byte left to the byte loop
      if ((reinterpret_cast<uintptr_t>(vb) & 3) == 0) {
        const uint32_t nw = nbytes >> 2;
        const uint32_t* vw = reinterpret_cast<const uint32_t*>(vb);
        for (uint32_t q = lane; q < nw; q += 32) {
          const uint32_t rem = tile.nrows - q * 32;
          z += __popc(~vw[q] & (rem >= 32 ? 0xffffffffu : ((1u << rem) - 1)));
        }
        j0 = nw << 2;
      }
      for (uint32_t j = j0 + lane; j < nbytes; j += 32) {
        const uint32_t rem = tile.nrows - j * 8;
        z += __popc(~(uint32_t)vb[j] & (rem >= 8 ? 0xffu : ((1u << rem) - 1)));
      }
      for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(kFull, z, o);
      if (lane == 0 && z) atomicAdd(&fd.nullcnt[(size_t)tile.batch * sd.n_array + a], z);
    }
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
// The plan: four small kernels between k_hash_count and k_scatter.
//   k_plan_prep  : per batch, which columns have nulls (hn) and input_has_null_ after the batch
//                  (ihn, sticky, quirk columns only, splitter.cc:878-886).
//   k_plan_rows  : one warp per partition restates the reference's per-pid buffer policy over
//                  the flush's batches, 32 batches per step: a warp scan of the row counts, then
//                  only the batches where the policy acts (allocation or a cut) are visited one
//                  by one, found with a ballot on "rows so far + count > capacity".  Writes the
//                  flush-local row / validity-bit offsets of every (segment, partition), the
//                  emission records, and marks cuts in rec_idx[batch][p].
//   k_plan_bytes : one warp per (binary column, partition): flush-local and in-segment byte
//                  offsets by warp scans, restarting at the cuts.
//   k_plan_scan  : exclusive scans over partitions -> output region starts.
constexpr int kPlanRowsThreads = 128;

__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t x) {
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if ((int)lane_id() >= o) x += y;
  }
  return x;
}
__device__ __forceinline__ unsigned long long warp_or64(unsigned long long v) {
  const uint32_t lo = __reduce_or_sync(kFull, (uint32_t)v);
  const uint32_t hi = __reduce_or_sync(kFull, (uint32_t)(v >> 32));
  return ((unsigned long long)hi << 32) | lo;
}
__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src) {
  return __shfl_sync(kFull, v, src);
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_prep(const SchemaDesc sd, const FlushDesc fd) {
  __shared__ unsigned long long s_warp[kPlanThreads / 32];
  const int NB = fd.n_batches;
  const int A = sd.n_array;
  const int per = (NB + kPlanThreads - 1) / kPlanThreads;
  const int lo = threadIdx.x * per, hi = min(lo + per, NB);
  unsigned long long run = 0;
  for (int b = lo; b < hi; b++) {
    unsigned long long m = 0;
    for (int a = 0; a < A; a++)
      if (fd.nullcnt[(size_t)b * A + a]) m |= 1ull << a;
    fd.hn[b] = m;
    run |= m & sd.quirk_mask;
  }
  // exclusive OR-scan of the per-thread ORs across the block
  unsigned long long x = run;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, x, o);
    if ((int)lane_id() >= o) x |= y;
  }
  const int w = threadIdx.x >> 5;
  if (lane_id() == 31) s_warp[w] = x;
  __syncthreads();
  unsigned long long before = *fd.st_ihn;
  for (int i = 0; i < w; i++) before |= s_warp[i];
  before |= __shfl_up_sync(kFull, x, 1) * (lane_id() ? 1ull : 0ull);
  for (int b = lo; b < hi; b++) {
    before |= fd.hn[b] & sd.quirk_mask;
    fd.ihn[b] = before;
  }
  __syncthreads();
  if (threadIdx.x == kPlanThreads - 1) {
    unsigned long long all = *fd.st_ihn;
    for (int i = 0; i < kPlanThreads / 32; i++) all |= s_warp[i];
    *fd.st_ihn = all;
  }
}

__global__ void __launch_bounds__(kPlanRowsThreads) k_plan_rows(const SchemaDesc sd, const FlushDesc fd) {
  const int P = sd.P;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= P) return;  // whole warps exit together
  const int lane = lane_id();
  const int NB = fd.n_batches;
  const int rec_words = kEmitFixedWords + sd.n_str;
  uint32_t cap = fd.st_cap[p];
  uint32_t base = fd.st_base[p];
  unsigned long long hv = fd.st_hv[p];
  uint32_t frow = 0, vpos = 0, piece_start = 0;  // flush-local rows; piece_start = frow of the piece
  // software pipeline over chunks of 32 batches: while chunk j is resolved, the descriptors of
  // chunk j + 2 are loaded and the row counts of chunk j + 1 (whose descriptors arrived during
  // chunk j - 1)
  auto load_desc = [&](int b, BatchDesc& bd, unsigned long long& hn, unsigned long long& ihn) {
    if (b < NB) {
      bd = fd.batches[b];
      hn = fd.hn[b];
      ihn = fd.ihn[b];
    } else {
      bd = BatchDesc{0, 0, 0, 0};
      hn = ihn = 0;
    }
  };
  auto load_rows = [&](const BatchDesc& bd) {
    uint32_t c = 0;
    for (uint32_t t = bd.seg0; t < bd.seg0 + bd.nsegs; t++) c += fd.cnt[(size_t)t * P + p];
    return c;
  };
  BatchDesc bd_c, bd_x, bd_y;
  unsigned long long hn_c, ihn_c, hn_x, ihn_x, hn_y, ihn_y;
  load_desc(lane, bd_c, hn_c, ihn_c);
  load_desc(lane + 32, bd_x, hn_x, ihn_x);
  uint32_t c_c = load_rows(bd_c);
  for (int b0 = 0; b0 < NB; b0 += 32) {
    const int b = b0 + lane;
    const bool active = b < NB;
    const BatchDesc bd = bd_c;
    const uint32_t c = c_c;
    const unsigned long long hn_l = hn_c, ihn_l = ihn_c;
    load_desc(b + 64, bd_y, hn_y, ihn_y);
    const uint32_t c_x = load_rows(bd_x);
    const uint32_t X = warp_incl_sum(c);
    const uint32_t Xex = X - c;
    const uint32_t total = __shfl_sync(kFull, X, 31);
    // events (allocation or cut) in lane order; state (cap, base_ref, hv) is warp-uniform.
    // base before lane l's rows = base_ref + (Xex[l] - Xex[ref]).
    int ref = 0, from = 0;
    uint32_t base_ref = base, pad = 0, my_pad = 0, rec = 0;
    for (;;) {
      const uint32_t ref_x = __shfl_sync(kFull, Xex, ref);
      const bool cond = active && lane >= from && c > 0 &&
                        (cap == 0 || base_ref + (Xex - ref_x) + c > cap);
      const unsigned m = __ballot_sync(kFull, cond);
      if (m == 0) break;
      const int e = __ffs(m) - 1;
      // validity presence accumulated over the rows since the last event
      hv |= warp_or64((active && lane >= from && lane < e && c > 0) ? hn_l : 0ull);
      const uint32_t c_e = __shfl_sync(kFull, c, e);
      const uint32_t xe = __shfl_sync(kFull, Xex, e);
      const uint32_t S_e = __shfl_sync(kFull, bd.split_size, e);
      const unsigned long long hn_e = shfl64(hn_l, e), ihn_e = shfl64(ihn_l, e);
      uint32_t base_e = base_ref + (xe - ref_x);
      if (lane == e) fd.call_flags[b] = 1u;
      if (cap == 0) {
        // first allocation: AllocatePartitionBuffers(max(S, cnt))
        cap = max(S_e, c_e);
        hv = ihn_e;
      } else {
        const uint32_t ns = max(S_e, c_e);
        if (base_e > 0) {
          // CacheRecordBatch: the pending rows become one record batch
          uint32_t idx = 0;
          if (lane == 0) idx = atomicAdd(fd.emit_count, 1u);
          idx = __shfl_sync(kFull, idx, 0);
          const uint32_t frow_e = frow + xe;
          if (idx < fd.emit_cap) {
            if (lane == 0) {
              uint32_t* r = fd.emit + (size_t)idx * rec_words;
              r[0] = (uint32_t)p;
              r[1] = frow_e;
              r[2] = base_e;
              r[3] = (uint32_t)hv;
              r[4] = (uint32_t)(hv >> 32);
            }
            if (lane == e) rec = idx + 1;
          } else if (lane == 0) {
            atomicOr(fd.err, kErrEmitOverflow);
          }
          // the next piece of validity bits starts on a 64-bit boundary
          if (frow_e > piece_start) {
            const uint32_t v = vpos + xe + pad;
            pad += ((v + 63u) & ~63u) - v;
          }
          piece_start = frow_e;
          base_e = 0;
        }
        if (!sd.prefer_spill || ns > cap) {
          // buffers reset and reallocated: validity presence restarts from input_has_null_
          hv = ihn_e;
          cap = ns;
        }
      }
      hv |= hn_e;  // SplitValidityBuffer: validity for every pid with rows in the batch
      if (lane >= e) my_pad = pad;
      ref = e;
      from = e + 1;
      base_ref = base_e;
    }
    hv |= warp_or64((active && lane >= from && c > 0) ? hn_l : 0ull);
    if (active && c > 0) {
      uint32_t fr = frow + Xex, vp = vpos + Xex + my_pad;
      for (uint32_t t = bd.seg0; t < bd.seg0 + bd.nsegs; t++) {
        const size_t ti = (size_t)t * P + p;
        const uint32_t ct = bd.nsegs == 1 ? c : fd.cnt[ti];  // a batch's only segment has its rows
        fd.cnt[ti] = fr;
        fd.vpos[ti] = vp;
        fr += ct;
        vp += ct;
      }
    }
    if (active) fd.rec_idx[(size_t)b * P + p] = rec;
    const uint32_t ref_x = __shfl_sync(kFull, Xex, ref);
    base = base_ref + (total - ref_x);
    frow += total;
    vpos += total + pad;
    bd_c = bd_x;
    hn_c = hn_x;
    ihn_c = ihn_x;
    c_c = c_x;
    bd_x = bd_y;
    hn_x = hn_y;
    ihn_x = ihn_y;
  }
  if (lane == 0) {
    fd.st_cap[p] = cap;
    fd.st_base[p] = base;
    fd.st_hv[p] = hv;
    const uint32_t vb = frow > piece_start ? ((vpos + 63u) & ~63u) : vpos;
    fd.rows_f[p] = frow;
    fd.vbits_f[p] = vb;
    fd.pstart[p] = frow;
    fd.vstart[p] = vb;
  }
}

__global__ void __launch_bounds__(kPlanRowsThreads) k_plan_bytes(const SchemaDesc sd, const FlushDesc fd) {
  const int P = sd.P;
  const int nstr = sd.n_str;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= nstr * P) return;
  const int k = wid / P, p = wid % P;
  const int lane = lane_id();
  const int T = fd.n_segs;
  const int rec_words = kEmitFixedWords + nstr;
  uint32_t sb = fd.st_sb[(size_t)k * P + p];
  uint32_t fb = 0;
  // software pipeline over chunks of 32 segments: while chunk j is resolved, the segments and
  // byte counts of chunk j + 2 are loaded and the cut records of chunk j + 1 (whose segments
  // arrived during chunk j - 1)
  auto load_seg = [&](int t, SegDesc& td, uint32_t& bc) {
    if (t < T) {
      td = fd.segs[t];
      bc = fd.bcnt[((size_t)t * nstr + k) * P + p];
    } else {
      td = SegDesc{0, 1, 0, 0, 0, {0, 0, 0}};  // row0 != 0: no cut record
      bc = 0;
    }
  };
  auto load_rec = [&](const SegDesc& td) {
    return td.row0 == 0 ? fd.rec_idx[(size_t)td.batch * P + p] : 0u;
  };
  SegDesc td_c, td_x, td_y;
  uint32_t bc_c, bc_x, bc_y;
  load_seg(lane, td_c, bc_c);
  load_seg(lane + 32, td_x, bc_x);
  uint32_t rec_c = load_rec(td_c);
  for (int t0 = 0; t0 < T; t0 += 32) {
    const int t = t0 + lane;
    const uint32_t bc = bc_c, rec = rec_c;
    load_seg(t + 64, td_y, bc_y);
    const uint32_t rec_x = load_rec(td_x);
    const uint32_t X = warp_incl_sum(bc);
    const uint32_t fb_l = fb + X - bc;
    // the last cut at or before this tile
    int last = rec ? lane : -1;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, last, o);
      if (lane >= o) last = max(last, y);
    }
    const uint32_t fb_last = __shfl_sync(kFull, fb_l, last < 0 ? 0 : last);
    const uint32_t sb_l = last < 0 ? sb + (fb_l - fb) : fb_l - fb_last;
    if (t < T) {
      if (rec) fd.emit[(size_t)(rec - 1) * rec_words + kEmitFixedWords + k] = fb_l;
      const size_t ix = ((size_t)t * nstr + k) * P + p;
      fd.bcnt[ix] = fb_l;
      fd.sbyte[ix] = sb_l;
    }
    const uint32_t total = __shfl_sync(kFull, X, 31);
    const int last31 = __shfl_sync(kFull, last, 31);
    const uint32_t fb_last31 = __shfl_sync(kFull, fb_l, last31 < 0 ? 0 : last31);
    sb = last31 < 0 ? sb + total : (fb + total) - fb_last31;
    fb += total;
    bc_c = bc_x;
    rec_c = rec_x;
    td_x = td_y;
    bc_x = bc_y;
  }
  if (lane == 0) {
    fd.st_sb[(size_t)k * P + p] = sb;
    fd.bytes_f[(size_t)k * P + p] = fb;
    fd.cstart[(size_t)k * P + p] = fb;
  }
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_scan(const SchemaDesc sd, const FlushDesc fd) {
  __shared__ uint32_t scan_scratch[33];
  const int P = sd.P;
  block_exscan<kPlanThreads>(fd.pstart, P, scan_scratch);
  block_exscan<kPlanThreads>(fd.vstart, P, scan_scratch);
  for (int k = 0; k < sd.n_str; k++) block_exscan<kPlanThreads>(fd.cstart + (size_t)k * P, P, scan_scratch);
}

// =======================================================================================
// k_scatter: one CTA per tile.
//
//   1. stable LSD radix sort of the tile's partition ids in shared memory (8-bit digits,
//      per-warp digit counts, one pass for P <= 256, two otherwise) -> sorted position j holds
//      source row ps[j]; rows of one partition form a run in input order
//   2. per sorted row: destination row (partition start + flush-local offset + rank in run)
//      and destination validity bit
//   3. column by column: the tile's slice of the column (values / offsets, and its validity
//      bits) is brought into shared memory by TMA bulk copies (cp.async.bulk, completion on an
//      mbarrier), double-buffered so the next column streams in while this one is scattered;
//      rows are then gathered from shared memory and written in sorted order, so the stores of
//      a run are contiguous.  Validity and bool bits start as 0xff-filled words; the zeros of the
//      tile (null rows, false values) are visited in source order and cleared by atomicAnd.
//      Characters of a binary column are copied one string per lane with aligned 32-bit
//      destination words built by funnel shifts from aligned source words.
namespace {
constexpr int kW = kScatterThreads / 32;
constexpr int kConsumers = kScatterThreads;          // threads that scatter; one more warp issues copies
constexpr int kScatterBlock = kConsumers + 32;
constexpr int kSlots = 4;                            // column slices in flight
constexpr int kStageBytes = kTileRows * 8 + 32;      // one 8-byte column slice, granule-aligned
constexpr int kStageValid = kTileRows / 8 + 32;      // its validity bits, granule-aligned
constexpr int kStageSlot = kStageBytes + kStageValid;
constexpr int kCharStage = 32768;                    // largest character slice that is staged
constexpr int kCharRegion = kCharStage + 64;         // + granule ends + read slack of the copy
constexpr uint32_t kSpinLimit = 1u << 26;

// Barrier of the scattering threads (the issuing warp never joins it).
__device__ __forceinline__ void csync() { group_sync<kConsumers, 1>(); }

// One stable LSD pass over 8 bits of the keys.  Warp w takes positions [w * seg, (w + 1) * seg);
// its keys, payloads and match masks stay in registers between the counting and the scatter.
constexpr int kSortIters = kTileRows / (kW * 32);  // 32-row groups per warp
__device__ void radix_pass(const uint16_t* kin, const uint16_t* pin, uint16_t* kout,
                           uint16_t* pout, int n, int shift, int ndig, uint16_t* wcnt, uint32_t* off,
                           uint32_t* scratch, uint32_t* first = nullptr) {
  // ndig: digit values that occur (keys < P), so only kW * ndig counters are scanned
  const int w = threadIdx.x >> 5;
  const int seg = ((n + kW * 32 - 1) / (kW * 32)) * 32;
  for (int i = threadIdx.x; i < kW * 256; i += kConsumers) wcnt[i] = 0;
  csync();
  uint16_t kv[kSortIters], pv[kSortIters];
  unsigned pe[kSortIters];
#pragma unroll
  for (int it = 0; it < kSortIters; it++) {
    const int c = it * 32;
    const int i = w * seg + c + lane_id();
    const bool act = c < seg && i < n;
    const unsigned m = __ballot_sync(kFull, act);
    kv[it] = 0;
    pv[it] = 0;
    pe[it] = 0;
    if (act) {
      kv[it] = kin[i];
      pv[it] = pin[i];
      const unsigned d = (kv[it] >> shift) & 255u;
      pe[it] = __match_any_sync(m, d);
      if ((int)lane_id() == __ffs(pe[it]) - 1) wcnt[w * 256 + d] += (uint16_t)__popc(pe[it]);
    }
    __syncwarp();
  }
  csync();
  // One digit per thread (ndig <= 256 threads): its count in each warp, an exclusive scan of the
  // digit totals over the block (one barrier), then its offset in each warp's part of the
  // output; `first` gets each digit's first sorted position, then n.
  {
    static_assert(kConsumers >= 256, "a thread per digit");
    const int d = threadIdx.x;
    uint32_t cw[kW];
    uint32_t tot = 0;
#pragma unroll
    for (int ww = 0; ww < kW; ww++) {
      cw[ww] = d < ndig ? wcnt[ww * 256 + d] : 0u;
      tot += cw[ww];
    }
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if ((int)lane_id() >= o) x += y;
    }
    if (lane_id() == 31) scratch[w] = x;
    csync();
    uint32_t base = x - tot;
    for (int ww = 0; ww < w; ww++) base += scratch[ww];
    if (d < ndig) {
      uint32_t run = base;
#pragma unroll
      for (int ww = 0; ww < kW; ww++) {
        off[d * kW + ww] = run;
        run += cw[ww];
      }
      if (first != nullptr) first[d] = base;
    }
    if (first != nullptr && d == 0) first[ndig] = (uint32_t)n;
    csync();  // the offsets are complete before the scatter below moves them
  }
#pragma unroll
  for (int it = 0; it < kSortIters; it++) {
    const int c = it * 32;
    const bool act = c < seg && w * seg + c + (int)lane_id() < n;
    const unsigned d = (kv[it] >> shift) & 255u;
    if (act) {
      const unsigned rank = __popc(pe[it] & ((1u << lane_id()) - 1));
      const uint32_t pos = off[d * kW + w] + rank;
      kout[pos] = kv[it];
      pout[pos] = pv[it];
    }
    __syncwarp();
    if (act && (int)lane_id() == __ffs(pe[it]) - 1) off[d * kW + w] += __popc(pe[it]);
    __syncwarp();
  }
  csync();
}

// ---- mbarrier + bulk copy (TMA) helpers -------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// 4-byte asynchronous global -> shared copies (no register holds the value in flight)
__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Bounded wait for phase `parity` of `bar`; false when `limit` polls ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kSpinLimit) {
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// A staged piece keeps the source's alignment phase: the aligned 16-byte granules covering
// [src, src + bytes) are copied by one bulk copy to a 16-byte aligned `dst_base`, so source byte x
// lands at dst_base + (x - (src & ~15)) and `src` itself at staged_ptr(dst_base, src).  The granules
// around a valid byte never leave its page, so the few extra bytes read at either end are always
// readable; they are never used.
__device__ __forceinline__ uint32_t super_bytes(const uint8_t* src, uint32_t bytes) {
  if (src == nullptr || bytes == 0) return 0;
  const uintptr_t lo = reinterpret_cast<uintptr_t>(src) & ~uintptr_t(15);
  const uintptr_t hi = (reinterpret_cast<uintptr_t>(src) + bytes + 15) & ~uintptr_t(15);
  return (uint32_t)(hi - lo);
}
__device__ __forceinline__ const uint8_t* staged_ptr(const uint8_t* dst_base, const uint8_t* src) {
  return dst_base + (reinterpret_cast<uintptr_t>(src) & 15);
}
__device__ __forceinline__ void stage_super(uint8_t* dst_base, const uint8_t* src, uint32_t super,
                                            uint64_t* bar) {
  if (super) bulk_g2s(dst_base, reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(src) & ~uintptr_t(15)),
                      super, bar);
}

// Source word at `a` (4-byte aligned); bytes outside [lo, hi) read as 0 and are never stored.
__device__ __forceinline__ uint32_t load_word(uintptr_t a, uintptr_t lo, uintptr_t hi) {
  if (a >= lo && a + 4 <= hi) return *reinterpret_cast<const uint32_t*>(a);
  uint32_t v = 0;
  for (int t = 0; t < 4; t++)
    if (a + t >= lo && a + t < hi) v |= (uint32_t)(*reinterpret_cast<const uint8_t*>(a + t)) << (8 * t);
  return v;
}

// One string: `len` bytes from `src` to `dst`.  Destination words are 4-byte aligned; each is
// built by a funnel shift of two aligned source words.  Eight destination words are produced
// per step from nine source words loaded up front, so a short string costs one memory latency
// rather than one per word.  Only bytes inside [buf_lo, buf_hi) of the source are read and only
// [dst, dst + len) is written.
__device__ __forceinline__ void copy_string(uint8_t* dst, const uint8_t* src, uint32_t len,
                                            uintptr_t buf_lo, uintptr_t buf_hi) {
  if (len == 0) return;
  const uintptr_t d = reinterpret_cast<uintptr_t>(dst);
  const uintptr_t dw0 = d & ~uintptr_t(3);
  const int nwd = (int)((((d + len - 1) & ~uintptr_t(3)) - dw0) >> 2) + 1;
  // source address of byte 0 of destination word 0
  const uintptr_t bs = reinterpret_cast<uintptr_t>(src) - (d - dw0);
  const uint32_t sh = (uint32_t)(bs & 3) * 8;
  const uintptr_t sw0 = bs & ~uintptr_t(3);
  const uintptr_t lo = reinterpret_cast<uintptr_t>(src) > buf_lo ? reinterpret_cast<uintptr_t>(src) : buf_lo;
  const uintptr_t hi = reinterpret_cast<uintptr_t>(src) + len < buf_hi ? reinterpret_cast<uintptr_t>(src) + len : buf_hi;
  for (int g = 0; g < nwd; g += 8) {
    uint32_t W[9];
#pragma unroll
    for (int q = 0; q < 9; q++) W[q] = (g + q <= nwd) ? load_word(sw0 + 4 * (uintptr_t)(g + q), lo, hi) : 0u;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (g + q >= nwd) break;
      const uint32_t v = sh ? __funnelshift_r(W[q], W[q + 1], sh) : W[q];
      const uintptr_t A = dw0 + 4 * (uintptr_t)(g + q);
      if (A >= d && A + 4 <= d + len) {
        *reinterpret_cast<uint32_t*>(A) = v;
      } else {
        for (int t = 0; t < 4; t++)
          if (A + t >= d && A + t < d + len) *reinterpret_cast<uint8_t*>(A + t) = (uint8_t)(v >> (8 * t));
      }
    }
  }
}

__device__ __forceinline__ uint32_t lds32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ uint32_t lds8(uint32_t addr) {
  uint16_t v;
  asm volatile("ld.shared.u8 %0, [%1];" : "=h"(v) : "r"(addr));
  return v;
}

// Bytes [lo, hi) of word `w` to the 4-byte aligned `p`: a byte at an odd start, then a halfword,
// then a last byte (at most two stores).
__device__ __forceinline__ void store_word_part(uint8_t* p, uint32_t w, uint32_t lo, uint32_t hi) {
  uint32_t x = lo;
  if (x & 1) {
    p[x] = (uint8_t)(w >> (8 * x));
    x++;
  }
  if (x + 2 <= hi) {
    *reinterpret_cast<uint16_t*>(p + x) = (uint16_t)(w >> (8 * x));
    x += 2;
  }
  if (x < hi) p[x] = (uint8_t)(w >> (8 * x));
}

// One string whose source bytes are in shared memory (shared address `src`): `len` bytes to
// global `dst`, written in the aligned 4-byte words of the destination: whole words as 16-byte
// stores of four, with a word and / or an 8-byte pair before them up to that alignment and after
// them for the rest.  Every destination word is a funnel shift of two aligned
// source words (one shift for the whole string), loaded as a stream; the first and last words,
// when the string covers them only in part, are stored as a byte and / or a halfword.  The aligned source words may reach 6 bytes before `src` and 7 past
// `src + len`: the staging buffer keeps that slack, and those bytes are never stored.
__device__ __forceinline__ void copy_string_smem(uint8_t* dst, uint32_t src, uint32_t len) {
  if (len <= 1) {  // empty, or one character (flag-like columns)
    if (len) dst[0] = (uint8_t)lds8(src);
    return;
  }
  const uintptr_t d = reinterpret_cast<uintptr_t>(dst);
  const uint32_t ph = (uint32_t)(d & 3);
  const uint32_t a = src - ph;  // source byte that maps to the first destination word
  uint32_t sb = a & ~3u;
  const uint32_t sh = (a & 3) * 8;
  uint8_t* X = dst - ph;
  uint32_t lo = lds32(sb);
  uint32_t rem = len;
  if (ph) {  // the string starts inside its first destination word
    const uint32_t hi = lds32(sb + 4);
    const uint32_t e = min(4u, ph + len);
    store_word_part(X, __funnelshift_r(lo, hi, sh), ph, e);
    rem -= e - ph;
    X += 4;
    sb += 4;
    lo = hi;
  }
  uint32_t* dw = reinterpret_cast<uint32_t*>(X);
  const uint32_t nw = rem >> 2;
  uint32_t k = 0;
  // up to 16-byte alignment: a word, then a pair
  if (nw > k && (reinterpret_cast<uintptr_t>(dw + k) & 4)) {
    const uint32_t hi = lds32(sb + 4 * k + 4);
    dw[k] = __funnelshift_r(lo, hi, sh);
    lo = hi;
    k += 1;
  }
  if (nw >= k + 2 && (reinterpret_cast<uintptr_t>(dw + k) & 8)) {
    const uint32_t w1 = lds32(sb + 4 * k + 4), w2 = lds32(sb + 4 * k + 8);
    *reinterpret_cast<uint2*>(dw + k) = make_uint2(__funnelshift_r(lo, w1, sh), __funnelshift_r(w1, w2, sh));
    lo = w2;
    k += 2;
  }
  for (; k + 4 <= nw; k += 4) {  // four source words loaded before one 16-byte store
    const uint32_t w1 = lds32(sb + 4 * k + 4), w2 = lds32(sb + 4 * k + 8);
    const uint32_t w3 = lds32(sb + 4 * k + 12), w4 = lds32(sb + 4 * k + 16);
    *reinterpret_cast<uint4*>(dw + k) = make_uint4(__funnelshift_r(lo, w1, sh), __funnelshift_r(w1, w2, sh),
                                                   __funnelshift_r(w2, w3, sh), __funnelshift_r(w3, w4, sh));
    lo = w4;
  }
  if (k + 2 <= nw) {
    const uint32_t w1 = lds32(sb + 4 * k + 4), w2 = lds32(sb + 4 * k + 8);
    *reinterpret_cast<uint2*>(dw + k) = make_uint2(__funnelshift_r(lo, w1, sh), __funnelshift_r(w1, w2, sh));
    lo = w2;
    k += 2;
  }
  if (k < nw) {
    const uint32_t hi = lds32(sb + 4 * k + 4);
    dw[k] = __funnelshift_r(lo, hi, sh);
    lo = hi;
  }
  if (rem & 3) {  // the string ends inside its last destination word
    const uint32_t hi = lds32(sb + 4 * nw + 4);
    store_word_part(reinterpret_cast<uint8_t*>(dw + nw), __funnelshift_r(lo, hi, sh), 0, rem & 3);
  }
}

// Rows a thread handles in a tile: j = threadIdx.x + u * kScatterThreads, u < kRowsPerThread.
// Loops over them load everything first and store afterwards, so the shared-memory loads of
// all rows are in flight together instead of each waiting behind the previous row's store.
constexpr int kRowsPerThread = kTileRows / kScatterThreads;
static_assert(kRowsPerThread * kScatterThreads == kTileRows, "tile rows per thread");

// One fixed-width column of the tile: value of source row sr[u] to destination row dr[u] (the
// thread's sorted positions, held in registers for every column of the tile).
template <typename V>
__device__ __forceinline__ void gather_rows(V* out, const V* src, const uint32_t* sr,
                                            const uint32_t* dr, int n) {
  V v[kRowsPerThread];
  uint32_t d[kRowsPerThread];
#pragma unroll
  for (int u = 0; u < kRowsPerThread; u++) {
    const int j = threadIdx.x + u * kScatterThreads;
    if (j < n) {
      d[u] = dr[u];
      v[u] = src[sr[u]];
    }
  }
#pragma unroll
  for (int u = 0; u < kRowsPerThread; u++)
    if (threadIdx.x + u * kScatterThreads < n) out[d[u]] = v[u];
}

// Clears, at its destination bit, the bit of every source row of the tile whose bit in `bits`
// is 0 (destination words start 0xff): the null rows of a validity bitmap, or the false values
// of a bool column.  Thread t < ceil(n / 8) takes source rows 8t .. 8t + 7 and visits only the
// zeros among them; `bits` is the shared address of the tile's staged bitmap (the bits past the
// tile's last row are slack of the stage and masked off), dbs[r] the destination bit of source
// row r.  Zeros of one destination word are cleared by separate atomicAnd calls.
__device__ __forceinline__ void scatter_zero_bits(uint32_t* words, uint32_t bits, const uint32_t* dbs, int n) {
  const int nb = (n + 7) >> 3;
  for (int t = threadIdx.x; t < nb; t += kConsumers) {
    uint32_t zeros = ~lds8(bits + t) & 0xffu;
    const int rem = n - 8 * t;
    if (rem < 8) zeros &= (1u << rem) - 1;
    while (zeros) {
      const int b = __ffs(zeros) - 1;
      zeros &= zeros - 1;
      const uint32_t pos = dbs[8 * t + b];
      atomicAnd(words + (pos >> 5), ~(1u << (pos & 31)));
    }
  }
}

// A list row's element validity: the zeros among source bits [e0, e0 + m) of `src` cleared at
// destination bits [d0, d0 + m) of `dst` (0xff-filled words), source read 32 bits at a time
// byte by byte (only bytes holding those bits).  Out of line: list columns only.
__device__ __noinline__ void clear_null_elements(uint32_t* dst, uint32_t d0, const uint8_t* src, uint32_t e0,
                                                 uint32_t m) {
  for (uint32_t x = 0; x < m; x += 32) {
    const uint32_t nb = min(32u, m - x);
    const uint32_t b = e0 + x;  // first source bit
    uint64_t w = 0;
    for (uint32_t y = b >> 3; y <= (b + nb - 1) >> 3; y++) w |= (uint64_t)src[y] << (8 * (y - (b >> 3)));
    uint32_t zeros = ~(uint32_t)(w >> (b & 7)) & (nb == 32 ? 0xffffffffu : (1u << nb) - 1u);
    while (zeros) {
      const uint32_t db = d0 + x + (uint32_t)(__ffs(zeros) - 1);
      zeros &= zeros - 1;
      atomicAnd(dst + (db >> 5), ~(1u << (db & 31)));
    }
  }
}

}  // namespace

// kLists: the schema has list columns (instantiated apart so the other schemas' code is unchanged)
template <bool kLists>
__global__ void __launch_bounds__(kScatterBlock, 2) k_scatter(const SchemaDesc sd, const FlushDesc fd) {
  extern __shared__ __align__(128) uint8_t ssm[];
  __shared__ uint32_t scratch[33];
  __shared__ uint32_t wtot[2][32];                 // warp totals of a binary column, by column parity
  __shared__ __align__(8) uint64_t full[kSlots];   // slice i landed (issuer: expect_tx)
  __shared__ __align__(8) uint64_t empty[kSlots];  // slice i consumed (every scattering warp)
  __shared__ __align__(8) uint64_t cfull, cempty;  // the same for the character stage
  __shared__ ColPtr s_col[kMaxCols];               // this batch's columns, by array index
  __shared__ uint32_t s_nc[kMaxCols];              // their null counts in the batch
  __shared__ int2 s_cr[kMaxStrPlan];               // character range of the tile per binary column
  __shared__ uint32_t s_bad;
  // per column of the tile in processing order: x = its staged slice's offset in shared memory,
  // y = shared address of its staged validity bits, z = kind | width << 8 | staged characters
  // << 16 | validity to clear << 17 | binary column index << 24, w = array column
  __shared__ uint4 s_ct[kMaxCols];
  const int T = kTileRows;
  uint8_t* stage0 = ssm;                                         // [kSlots][kStageSlot]
  uint8_t* cstage = ssm + kSlots * kStageSlot;                   // [kCharRegion]
  uint16_t* kA = reinterpret_cast<uint16_t*>(cstage + kCharRegion);
  uint16_t* pA = kA + T;
  uint16_t* kB = pA + T;
  uint16_t* pB = kB + T;
  uint16_t* rs = pB + T;                                    // [T]
  uint32_t* S = reinterpret_cast<uint32_t*>(rs + T);        // [T + 1]
  uint32_t* rt0 = S + T + 1;                                // [T] run tables (at run starts)
  uint32_t* rt1 = rt0 + T;                                  // [T]
  uint16_t* wcnt = reinterpret_cast<uint16_t*>(rt1 + T);    // [kW * 256]
  uint32_t* nm2 = reinterpret_cast<uint32_t*>(wcnt + kW * 256);  // [T]
  uint32_t* nm3 = nm2 + T;                                         // [T]
  uint32_t* dbs = nm3 + T;                                         // [T] destination bit by source row
  // radix offsets while sorting: rs, S and the start of rt0 are written only after the sort
  uint32_t* roff = reinterpret_cast<uint32_t*>(rs);
  static_assert(kW * 256 * sizeof(uint32_t) <= sizeof(uint16_t) * kTileRows + 2 * sizeof(uint32_t) * kTileRows,
                "radix offsets fit over rs, S and rt0");
  // run metadata of the next binary column, by sorted position of the run start (S and wcnt
  // are free once the destinations are computed and the sort is done)
  uint32_t* nm0 = S;
  uint32_t* nm1 = reinterpret_cast<uint32_t*>(wcnt);
  static_assert(kW * 256 * sizeof(uint16_t) >= kTileRows * sizeof(uint32_t), "wcnt holds a row table");

  const TileDesc tile = fd.tiles[blockIdx.x];
  const int n = (int)tile.nrows;
  const int P = sd.P;
  const int nstr = sd.n_str;
  const int A = sd.n_array;
  const uint32_t row0 = tile.row0;
  {
    const ColPtr* cols = fd.cols + (size_t)tile.batch * sd.n_cols;
    if ((int)threadIdx.x < A) {
      s_col[threadIdx.x] = cols[sd.arr_col[threadIdx.x]];
      s_nc[threadIdx.x] = fd.nullcnt[(size_t)tile.batch * A + threadIdx.x];
    }
    if ((int)threadIdx.x < nstr) s_cr[threadIdx.x] = fd.crange[(size_t)blockIdx.x * nstr + threadIdx.x];
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kSlots; i++) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], kW);
    }
    mbar_init(&cfull, 1);
    mbar_init(&cempty, kW);
    // inputs rejected by k_hash_count: copy nothing (read once, so the whole block agrees)
    s_bad = (*reinterpret_cast<volatile int32_t*>(fd.err) & (kErrBadOffsets | kErrBadPid)) != 0;
    fence_mbar_init();
  }
  __syncthreads();  // the last barrier of the whole block: the issuing warp leaves early
  if (s_bad) return;

  // characters of binary column k are staged when the tile's slice fits the stage
  auto chars_staged = [&](int k) {
    const int32_t len = s_cr[k].y - s_cr[k].x;
    return len > 0 && len <= kCharStage;
  };
  // (the element bits of a list of bool elements are not staged: they are read from global memory)
  auto staged_binary = [&](int a) {
    return sd.arr_kind[a] == COL_BINARY && !(kLists && ((sd.listbit_mask >> a) & 1ull)) && chars_staged(sd.arr_str[a]);
  };

  // Polls of a wait for data or for a free slot before the block gives up (a test lowers it to
  // make the waits run out); waits for copies already in flight always use kSpinLimit.
  const uint32_t lim = fd.spin_limit ? fd.spin_limit : kSpinLimit;
  volatile uint32_t* vbad = &s_bad;

  // ---- issuing warp: lane 0 streams the column slices, lane 1 the character slices ----------
  // Once a scattering warp has given up on a slice (s_bad, written before that warp releases the
  // slot), nothing more is issued: the slot's last copy may still be landing.
  if (threadIdx.x >= kConsumers) {
    const int lane = threadIdx.x - kConsumers;
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < A; i++) {
        if (i >= kSlots && !mbar_wait(&empty[i % kSlots], (uint32_t)((i / kSlots - 1) & 1), lim)) {
          atomicOr(fd.err, kErrTimeout);
          break;
        }
        if (*vbad) break;
        const int a = sd.order[i];
        const ColPtr c = s_col[a];
        const int kind = sd.arr_kind[a];
        const uint8_t* vsrc = nullptr;
        uint32_t vbytes = 0;
        if (kind == COL_FIXED && sd.arr_width[a] <= 8) {
          vsrc = c.values + (size_t)row0 * sd.arr_width[a];
          vbytes = (uint32_t)n * sd.arr_width[a];
        } else if (kind == COL_BOOL) {
          vsrc = c.values + (row0 >> 3);
          vbytes = (uint32_t)(n + 7) >> 3;
        } else if (kind == COL_BINARY) {  // offsets of 4 or 8 bytes (arr_width)
          vsrc = reinterpret_cast<const uint8_t*>(c.offsets) + (size_t)row0 * sd.arr_width[a];
          vbytes = (uint32_t)(n + 1) * sd.arr_width[a];
        }
        const uint8_t* bsrc = nullptr;
        uint32_t bbytes = 0;
        if (c.validity != nullptr && s_nc[a] != 0 && fd.out_valid[a] != nullptr) {
          bsrc = c.validity + (row0 >> 3);
          bbytes = (uint32_t)(n + 7) >> 3;
        }
        const uint32_t vs = super_bytes(vsrc, vbytes), bs = super_bytes(bsrc, bbytes);
        uint8_t* dst = stage0 + (i % kSlots) * kStageSlot;
        fence_proxy_async();  // the scattering threads' generic reads of the slot come first
        mbar_expect_tx(&full[i % kSlots], vs + bs);
        stage_super(dst, vsrc, vs, &full[i % kSlots]);
        stage_super(dst + kStageBytes, bsrc, bs, &full[i % kSlots]);
        issued = i + 1;
      }
      // leave no copy in flight into this CTA's shared memory: wait (bounded) for the last
      // phase issued on every slot
      for (int i = max(0, issued - kSlots); i < issued; i++)
        mbar_wait(&full[i % kSlots], (uint32_t)((i / kSlots) & 1));
    } else if (lane == 1) {
      uint32_t uses = 0;
      for (int i = 0; i < A; i++) {
        const int a = sd.order[i];
        if (!staged_binary(a)) continue;
        if (uses > 0 && !mbar_wait(&cempty, (uses - 1) & 1, lim)) {
          atomicOr(fd.err, kErrTimeout);
          break;
        }
        if (*vbad) break;
        const int k = sd.arr_str[a];
        const uint8_t* src = s_col[a].values + s_cr[k].x;
        const uint32_t sb = super_bytes(src, (uint32_t)(s_cr[k].y - s_cr[k].x));
        fence_proxy_async();
        mbar_expect_tx(&cfull, sb);
        stage_super(cstage, src, sb, &cfull);
        uses++;
      }
      if (uses > 0) mbar_wait(&cfull, (uses - 1) & 1);
    }
    return;
  }

  // ---- scattering threads --------------------------------------------------------------------
  for (int i = threadIdx.x; i < A; i += kConsumers) {
    const int a = sd.order[i];
    const int kind = sd.arr_kind[a];
    const int w = sd.arr_width[a];
    const ColPtr c = s_col[a];
    const uint8_t* slot_base = stage0 + (i % kSlots) * kStageSlot;
    const uint8_t* stg = slot_base;  // staged values / bits / offsets, at the source's phase
    if (kind == COL_FIXED && w <= 8) stg = staged_ptr(slot_base, c.values + (size_t)row0 * w);
    else if (kind == COL_BOOL) stg = staged_ptr(slot_base, c.values + (row0 >> 3));
    else if (kind == COL_BINARY) stg = staged_ptr(slot_base, reinterpret_cast<const uint8_t*>(c.offsets) + (size_t)row0 * w);
    const bool vwork = c.validity != nullptr && s_nc[a] != 0 && fd.out_valid[a] != nullptr;
    const uint32_t vb = vwork ? smem_addr(staged_ptr(slot_base + kStageBytes, c.validity + (row0 >> 3))) : 0u;
    s_ct[i] = make_uint4((uint32_t)(stg - ssm), vb,
                         (uint32_t)kind | ((uint32_t)w << 8) | ((uint32_t)staged_binary(a) << 16) |
                             ((uint32_t)vwork << 17) | ((uint32_t)(kind == COL_BINARY ? sd.arr_str[a] : 0) << 24),
                         (uint32_t)a);
  }
  // destination row / validity bit of a partition's first row in the tile: its segment offset
  // from the plan + rows from the segment's earlier tiles
  const size_t tp = (size_t)tile.seg * P;
  const bool has_pre = tile.tseg > 0;
  // Up to 256 partitions (one radix pass): thread p reads partition p's entries now, so the
  // loads are in flight during the sort, and the sort itself gives each partition's first sorted
  // position (no scan for the run starts).
  const bool small = P <= 256;
  uint32_t t_ps = 0, t_cnt = 0, t_pre = 0, t_vs = 0, t_vp = 0;
  if (small && (int)threadIdx.x < P) {
    const int p = threadIdx.x;
    t_ps = fd.pstart[p];
    t_cnt = fd.cnt[tp + p];
    t_pre = has_pre ? fd.tilepre[(size_t)blockIdx.x * P + p] : 0u;
    t_vs = fd.vstart[p];
    t_vp = fd.vpos[tp + p];
  }
  for (int j = threadIdx.x; j < n; j += kConsumers) {
    kA[j] = fd.pids[tile.frow0 + j];
    pA[j] = (uint16_t)j;
  }
  csync();
  uint32_t* first = nm2;  // [P + 1] (nm2 is free until the run metadata of the binary columns)
  radix_pass(kA, pA, kB, pB, n, 0, min(P, 256), wcnt, roff, scratch, small ? first : nullptr);
  uint16_t* ks = kB;
  uint16_t* ps = pB;
  uint32_t* dstrow = reinterpret_cast<uint32_t*>(kA);  // kA,pA are free after one pass
  if (!small) {
    radix_pass(kB, pB, kA, pA, n, 8, ((P - 1) >> 8) + 1, wcnt, roff, scratch);
    ks = kA;
    ps = pA;
    dstrow = reinterpret_cast<uint32_t*>(kB);
  }

  // run starts: rs[j] = first sorted position with the same partition id; S / rt1 at a run
  // start: the run's destination row / validity bit minus that position
  if (small) {
    if ((int)threadIdx.x < P) {
      const int p = threadIdx.x;
      const uint32_t f = first[p];
      if (first[p + 1] > f) {  // partition p has rows in this tile
        S[f] = t_ps + t_cnt + t_pre - f;
        rt1[f] = t_vs + t_vp + t_pre - f;
      }
    }
    for (int j = threadIdx.x; j < n; j += kConsumers) rs[j] = (uint16_t)first[ks[j]];
    csync();
  } else {
    {
      const int per = (n + kConsumers - 1) / kConsumers;
      const int lo = threadIdx.x * per;
      const int hi = min(lo + per, n);
      uint32_t mx = 0;
      for (int j = lo; j < hi; j++)
        if (j == 0 || ks[j] != ks[j - 1]) mx = j;
      uint32_t carry = block_exmax<kConsumers, 1>(mx, scratch);
      for (int j = lo; j < hi; j++) {
        if (j == 0 || ks[j] != ks[j - 1]) carry = j;
        rs[j] = (uint16_t)carry;
      }
    }
    csync();
    for (int j = threadIdx.x; j < n; j += kConsumers) {
      if (rs[j] == j) {
        const int p = ks[j];
        const uint32_t before = has_pre ? fd.tilepre[(size_t)blockIdx.x * P + p] : 0u;
        S[j] = fd.pstart[p] + fd.cnt[tp + p] + before - (uint32_t)j;
        rt1[j] = fd.vstart[p] + fd.vpos[tp + p] + before - (uint32_t)j;
      }
    }
    csync();
  }
  for (int j = threadIdx.x; j < n; j += kConsumers) {
    dstrow[j] = S[rs[j]] + (uint32_t)j;
    dbs[ps[j]] = rt1[rs[j]] + (uint32_t)j;
  }

  // Binary columns: thread t owns sorted positions t + u * kConsumers, u < kRowsPerThread.  The
  // run metadata of the next binary column (in-segment byte offset and destination byte of each
  // run that starts at an owned position) is copied asynchronously into nm0/nm1/nm2 one binary
  // column ahead, so its latency is hidden behind the columns processed in between; only the
  // owning thread reads it back.
  // Up to 256 partitions: thread p loads partition p's values instead (nmP[0..3][p]); after they
  // land the same thread turns them into the column's bases, so no other thread reads them.
  uint32_t* nmP = nm3;                 // [4][256] (nm3 is free after the destinations)
  uint32_t* baseP = rt0;               // [2 column parities][2][256] offset / character bases
  uint32_t* wexP = rt1;                // [2][256] prefix inside its 32-row block at the run start
  auto load_run_meta = [&](int i_from) {
    for (int i = i_from; i < A; i++) {
      const int a = sd.order[i];
      if (sd.arr_kind[a] != COL_BINARY) continue;
      const int k = sd.arr_str[a];
      const size_t tk = ((size_t)tile.seg * nstr + k) * P;
      const size_t tb = ((size_t)blockIdx.x * nstr + k) * P;
      const uint32_t* cst = fd.cstart + (size_t)k * P;
      if (small) {
        const int p = threadIdx.x;
        if (p < P) {
          cp_async4(&nmP[p], &fd.sbyte[tk + p]);
          cp_async4(&nmP[256 + p], &fd.bcnt[tk + p]);
          cp_async4(&nmP[512 + p], &cst[p]);
          if (has_pre) cp_async4(&nmP[768 + p], &fd.tilebpre[tb + p]);
        }
        cp_async_commit();
        return;
      }
#pragma unroll
      for (int u = 0; u < kRowsPerThread; u++) {
        const int j = threadIdx.x + u * kConsumers;
        if (j < n && rs[j] == j) {
          const int p = ks[j];
          cp_async4(&nm0[j], &fd.sbyte[tk + p]);
          cp_async4(&nm1[j], &fd.bcnt[tk + p]);
          cp_async4(&nm2[j], &cst[p]);
          if (has_pre) cp_async4(&nm3[j], &fd.tilebpre[tb + p]);
        }
      }
      cp_async_commit();
      return;
    }
  };
  csync();  // rs and the tables of the run starts are complete
  load_run_meta(0);
  uint32_t cuse = 0;  // staged character slices consumed

  // Warps run through fixed-width and bool columns at their own pace (the slots' mbarriers keep
  // the fastest within kSlots columns of the slowest); a binary column has two barriers of the
  // scattering threads, after its warp totals and after its run tables.  A wait that times out
  // marks the block bad: from then on columns are skipped, but every thread still reaches every
  // barrier (a binary column's skip decision is taken after its first barrier, so it is the same
  // in all threads).
  int nbin = 0;  // binary columns done (the parity of their warp-total buffer)
  // this thread's sorted positions: source row and destination row, held for every column
  uint32_t r_ps[kRowsPerThread], r_d[kRowsPerThread];
#pragma unroll
  for (int u = 0; u < kRowsPerThread; u++) {
    const int j = threadIdx.x + u * kConsumers;
    r_ps[u] = j < n ? ps[j] : 0u;
    r_d[u] = j < n ? dstrow[j] : 0u;
  }
  for (int i = 0; i < A; i++) {
    const uint4 ct = s_ct[i];
    const int a = (int)ct.w;
    const int slot = i % kSlots;
    const bool chars = (ct.z >> 16) & 1u;
    const int kind = (int)(ct.z & 255u);
    if (!*vbad) {
      bool ok = mbar_wait(&full[slot], (uint32_t)((i / kSlots) & 1), lim);
      if (chars) ok = mbar_wait(&cfull, cuse & 1, lim) && ok;
      if (!ok) {
        atomicOr(fd.err, kErrTimeout);
        *vbad = 1;
      }
    }
    const bool live = !*vbad;  // fixed / bool columns: this thread's view is enough
    if (live || kind == COL_BINARY) {
      const uint8_t* stg = ssm + ct.x;  // staged values / bits / offsets, at the source's phase
      // validity: clear the bits of null rows (destination words start 0xff)
      if (live && ((ct.z >> 17) & 1u)) scatter_zero_bits(fd.out_valid[a], ct.y, dbs, n);
      if (kind == COL_FIXED && live) {
        const int w = (int)((ct.z >> 8) & 255u);
        uint8_t* out = fd.out_values[a];
        if (w == 8) {
          gather_rows(reinterpret_cast<uint64_t*>(out), reinterpret_cast<const uint64_t*>(stg), r_ps, r_d, n);
        } else if (w == 4) {
          gather_rows(reinterpret_cast<uint32_t*>(out), reinterpret_cast<const uint32_t*>(stg), r_ps, r_d, n);
        } else if (w == 2) {
          gather_rows(reinterpret_cast<uint16_t*>(out), reinterpret_cast<const uint16_t*>(stg), r_ps, r_d, n);
        } else if (w == 1) {
          gather_rows(out, stg, r_ps, r_d, n);
        } else {  // 16-byte values are gathered straight from global memory
          const uint4* src = reinterpret_cast<const uint4*>(s_col[a].values) + row0;
          for (int j = threadIdx.x; j < n; j += kConsumers) reinterpret_cast<uint4*>(out)[dstrow[j]] = src[ps[j]];
        }
      } else if (kind == COL_BOOL && live) {
        scatter_zero_bits(fd.out_bits[a], smem_addr(stg), dbs, n);
      } else if (kind == COL_BINARY) {
        // every thread takes both barriers of a binary column; the lengths and their warp scans
        // read only the slot (in bounds whether or not its copy arrived), and after the first
        // barrier the block's state, the same in every thread, decides whether the rest runs
        const ColPtr c = s_col[a];
        // offsets of rows row0..row0+n, 4 or 8 bytes each (valid ones are below 2^31 either way)
        const bool off64 = ((ct.z >> 8) & 255u) == 8;
        const int32_t* oin = reinterpret_cast<const int32_t*>(stg);
        const int64_t* oin64 = reinterpret_cast<const int64_t*>(stg);
        // a list column: element offsets, elements of 1 << shift bytes; a null row has none
        const int shift = kLists ? sd.arr_shift[a] : 0;
        const bool list = kLists && ((sd.list_mask >> a) & 1ull);
        const uint32_t lvb = list && ((ct.z >> 17) & 1u) ? ct.y : 0u;  // staged row validity
        // lengths of the owned positions; exclusive prefix over the tile = the lengths of all
        // earlier rows u' < u of positions + this row's prefix, one fused warp scan per row u
        uint32_t len[kRowsPerThread], pre[kRowsPerThread], so[kRowsPerThread];  // so: source offset
#pragma unroll
        for (int u = 0; u < kRowsPerThread; u++) {
          const int j = threadIdx.x + u * kConsumers;
          len[u] = 0;
          so[u] = 0;
          if (j < n) {
            const int r = (int)r_ps[u];
            if (off64) {
              so[u] = (uint32_t)oin64[r];
              len[u] = (uint32_t)oin64[r + 1] - so[u];
            } else {
              so[u] = (uint32_t)oin[r] << shift;
              len[u] = ((uint32_t)oin[r + 1] << shift) - so[u];
              if (lvb && !((lds8(lvb + (r >> 3)) >> (r & 7)) & 1u)) len[u] = 0;
            }
          }
          pre[u] = len[u];
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) {
            const uint32_t y = __shfl_up_sync(kFull, pre[u], o);
            if ((int)lane_id() >= o) pre[u] += y;
          }
        }
        const int w = threadIdx.x >> 5;
        const int bb = nbin & 1;
        uint32_t* tot = wtot[bb];  // the previous binary column's totals may still be read
        if (lane_id() == 31) {
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) tot[u * kW + w] = pre[u];
        }
        if (small) {
          // before the one barrier of the column: partition p's bases (thread p, from its own
          // loads), the next binary column's loads, and at each run start the prefix inside its
          // 32-row block (every thread has finished the reads of these buffers two binary
          // columns back: it has passed the previous binary column's barrier)
          cp_async_wait_all();
          if ((int)threadIdx.x < P) {
            const int p = threadIdx.x;
            const uint32_t before = has_pre ? nmP[768 + p] : 0u;  // bytes from the segment's earlier tiles
            baseP[bb * 512 + p] = nmP[p] + before;
            baseP[bb * 512 + 256 + p] = nmP[512 + p] + nmP[256 + p] + before;
          }
          load_run_meta(i + 1);
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) {
            const int j = threadIdx.x + u * kConsumers;
            if (j < n && rs[j] == j) wexP[bb * 256 + ks[j]] = pre[u] - len[u];
          }
        }
        csync();
        const bool run = !*vbad;
        uint32_t excl = 0;
        if (run) {
          // the warp totals in (row, warp) order, one per lane: their exclusive scan is what all
          // earlier rows and this row's earlier warps hold (every warp scans them itself)
          static_assert(kRowsPerThread * kW == 32, "one warp total per lane");
          const uint32_t sv = tot[lane_id()];
          uint32_t incl = sv;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFull, incl, o);
            if ((int)lane_id() >= o) incl += y;
          }
          excl = incl - sv;
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) pre[u] = __shfl_sync(kFull, excl, u * kW + w) + pre[u] - len[u];
          if (!small) {
            // run tables at the run starts: destination of the run's first string and its offset
            // inside the partition's segment, both relative to the tile prefix (every thread has
            // finished the previous binary column's reads of them: it passed the barrier above)
            cp_async_wait_all();
#pragma unroll
            for (int u = 0; u < kRowsPerThread; u++) {
              const int j = threadIdx.x + u * kConsumers;
              if (j < n && rs[j] == j) {
                const uint32_t before = has_pre ? nm3[j] : 0u;  // bytes from the segment's earlier tiles
                rt0[j] = nm0[j] + before - pre[u];
                rt1[j] = nm2[j] + nm1[j] + before - pre[u];
              }
            }
            load_run_meta(i + 1);
          }
        }
        if (!small) csync();
        nbin++;
        if (run) {
        int32_t* ooff = reinterpret_cast<int32_t*>(fd.out_values[a]);
        uint8_t* ochars = fd.out_chars[a];
        uint32_t cd[kRowsPerThread];  // destination of each string in the column's characters
        {
          uint32_t d[kRowsPerThread], v[kRowsPerThread];
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) {
            const int j = threadIdx.x + u * kConsumers;
            if (small) {
              // the run start q's tile prefix: its block's exclusive prefix (lane u_q * kW + w_q
              // of every warp's scan) + the prefix inside the block published before the barrier
              const uint32_t q = j < n ? rs[j] : 0u;
              const uint32_t blk = __shfl_sync(kFull, excl, (int)((q >> 8) * kW + ((q & 255u) >> 5)));
              if (j < n) {
                const int p = ks[j];
                const uint32_t rel = pre[u] - blk - wexP[bb * 256 + p];  // bytes of the run before row j
                d[u] = r_d[u];
                v[u] = baseP[bb * 512 + p] + rel + len[u];
                cd[u] = baseP[bb * 512 + 256 + p] + rel;
              }
            } else if (j < n) {
              const int q = rs[j];
              d[u] = r_d[u];
              v[u] = rt0[q] + pre[u] + len[u];
              cd[u] = rt1[q] + pre[u];
            }
          }
          if (off64) {
#pragma unroll
            for (int u = 0; u < kRowsPerThread; u++)
              if (threadIdx.x + u * kConsumers < n) reinterpret_cast<int64_t*>(ooff)[d[u]] = (int64_t)v[u];
          } else {
#pragma unroll
            for (int u = 0; u < kRowsPerThread; u++)
              if (threadIdx.x + u * kConsumers < n) ooff[d[u]] = (int32_t)(v[u] >> shift);
          }
        }
        const int k = (int)(ct.z >> 24);
        if (kLists && ((sd.listbit_mask >> a) & 1ull)) {
          // bool elements: each row's element bits [so, so + len) to the bit region at cd (its
          // words start 0xff: the false ones are cleared); struct entries carry no values
          if (!((sd.nopay_mask >> a) & 1ull)) {
#pragma unroll
            for (int u = 0; u < kRowsPerThread; u++)
              if (threadIdx.x + u * kConsumers < n && len[u])
                clear_null_elements(reinterpret_cast<uint32_t*>(ochars), cd[u], c.values, so[u], len[u]);
          }
        } else if (chars) {
          // shared address of byte 0 of the column (offsets index from there)
          const uint32_t cbase = smem_addr(staged_ptr(cstage, c.values + s_cr[k].x)) - (uint32_t)s_cr[k].x;
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) {
            const int j = threadIdx.x + u * kConsumers;
            if (j < n) copy_string_smem(ochars + cd[u], cbase + so[u], len[u]);
          }
        } else {
          const uintptr_t buf_lo = reinterpret_cast<uintptr_t>(c.values);
          const uintptr_t buf_hi = buf_lo + c.values_bytes;
#pragma unroll
          for (int u = 0; u < kRowsPerThread; u++) {
            const int j = threadIdx.x + u * kConsumers;
            if (j < n) copy_string(ochars + cd[u], c.values + so[u], len[u], buf_lo, buf_hi);
          }
        }
        // a list column's element validity: the null elements of each row cleared at their
        // destination element (bits start 0xff), read 32 at a time from the batch's bitmap
        if constexpr (kLists) {
          if (list && c.child_validity != nullptr && fd.out_cvalid[a] != nullptr) {
#pragma unroll
            for (int u = 0; u < kRowsPerThread; u++)
              if (threadIdx.x + u * kConsumers < n && len[u])
                clear_null_elements(fd.out_cvalid[a], cd[u] >> shift, c.child_validity, so[u] >> shift,
                                    len[u] >> shift);
          }
        }
        }
      }
    }
    __syncwarp();  // the whole warp is done with the slice (and the character stage)
    if (lane_id() == 0) {
      mbar_arrive(&empty[slot]);
      if (chars) mbar_arrive(&cempty);
    }
    if (chars) cuse++;
  }
  cp_async_wait_all();  // no run-metadata copy is left in flight when the block exits
}

// =======================================================================================
// k_gather: host input buffers into device staging, read by the SMs straight from host memory
// over the coherent link.  Each CTA copies whole buffers, striding over the job list; `jobs`
// itself lives in pinned host memory.
// The host places each buffer in staging at its source's alignment phase (mod 16) whenever the
// source is aligned to its element width, so the body moves as aligned 16-byte words and only
// a head and a tail of < 16 bytes go byte by byte.  Other phase pairs fall back to 4-byte words
// or bytes.  Only [src, src + bytes) is read and [dst, dst + bytes) written.
template <typename V>
__device__ __forceinline__ void gather_words(const uint8_t* src, uint8_t* dst, uint64_t n) {
  constexpr uint32_t W = sizeof(V);
  const uint64_t lead = (W - (reinterpret_cast<uintptr_t>(src) & (W - 1))) & (W - 1);
  const uint64_t head = n < lead ? n : lead;
  if (threadIdx.x < head) dst[threadIdx.x] = src[threadIdx.x];
  const uint64_t nv = (n - head) / W;
  const V* sv = reinterpret_cast<const V*>(src + head);
  V* dv = reinterpret_cast<V*>(dst + head);
  constexpr int U = 4;  // loads in flight per thread
  uint64_t i = threadIdx.x;
  for (; i + (U - 1) * 256 < nv; i += U * 256) {
    V v[U];
#pragma unroll
    for (int u = 0; u < U; u++) v[u] = sv[i + u * 256];
#pragma unroll
    for (int u = 0; u < U; u++) dv[i + u * 256] = v[u];
  }
  for (; i < nv; i += 256) dv[i] = sv[i];
  for (uint64_t j = head + nv * W + threadIdx.x; j < n; j += 256) dst[j] = src[j];
}

__global__ void __launch_bounds__(256) k_gather(const HostCopy* __restrict__ jobs, uint32_t n_jobs) {
  for (uint32_t b = blockIdx.x; b < n_jobs; b += gridDim.x) {
    const HostCopy job = jobs[b];
    const uintptr_t phase = reinterpret_cast<uintptr_t>(job.src) ^ reinterpret_cast<uintptr_t>(job.dst);
    if ((phase & 15) == 0) {
      gather_words<uint4>(job.src, job.dst, job.bytes);
    } else if ((phase & 3) == 0) {
      gather_words<uint32_t>(job.src, job.dst, job.bytes);
    } else {
      for (uint64_t j = threadIdx.x; j < job.bytes; j += 256) job.dst[j] = job.src[j];
    }
  }
}

// =======================================================================================
// k_nest_prep: the per-batch arrays of nested columns - row ranges composed through the offsets
// of every list / map on a node's path, and the lengths of binary / list / map entries - one
// job per block, striding.  Every read is checked against the entries of the array it reads;
// a failed check writes 0 and raises kErrBadOffsets (the pass then copies nothing).
__global__ void __launch_bounds__(256) k_nest_prep(const NestJob* __restrict__ jobs, uint32_t n_jobs,
                                                   int32_t* err) {
  for (uint32_t j = blockIdx.x; j < n_jobs; j += gridDim.x) {
    const NestJob& job = jobs[j];
    bool bad = false, span = false;
    if (job.kind == 0) {
      for (uint32_t r = threadIdx.x; r < job.n; r += blockDim.x) {
        int64_t x = r;
        for (uint32_t d = 0; d < job.depth; d++) {
          if (x < 0 || (uint64_t)x >= job.lim[d]) {
            bad = true;
            x = 0;
            break;
          }
          x = job.wide[d] ? static_cast<const int64_t*>(job.off[d])[x] : (int64_t) static_cast<const int32_t*>(job.off[d])[x];
        }
        if (x < 0 || x > INT32_MAX) {
          bad = true;
          x = 0;
        }
        job.out[r] = (int32_t)x;
      }
    } else {
      for (uint32_t i = threadIdx.x; i < job.n; i += blockDim.x) {
        int64_t len = 0;
        if ((uint64_t)i + 1 < job.lim[0]) {
          len = job.wide[0] ? static_cast<const int64_t*>(job.off[0])[i + 1] - static_cast<const int64_t*>(job.off[0])[i]
                            : (int64_t) static_cast<const int32_t*>(job.off[0])[i + 1] -
                                  static_cast<const int32_t*>(job.off[0])[i];
        } else {
          bad = true;
        }
        if (len < 0 || len > INT32_MAX) {
          bad = true;
          len = 0;
        }
        if (job.validity != nullptr) {
          if (i >= job.lim[1]) {  // beyond the validity buffer
            bad = true;
            len = 0;
          } else if (!((job.validity[i >> 3] >> (i & 7)) & 1)) {
            if (len != 0 && job.inner) span = true;
            len = 0;
          }
        }
        job.out[i] = (int32_t)len;
      }
    }
    if (bad) atomicOr(err, kErrBadOffsets);
    if (span) atomicOr(err, kErrNestSpan);
  }
}

// =======================================================================================
// launch helpers
cudaError_t launch_hash_count(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  const size_t sm = fd.hist_in_smem ? sizeof(uint32_t) * sd.P * (1 + sd.n_str) : 0;
  const bool lists = sd.list_mask != 0;
  if (sm > 48 * 1024) {
    cudaError_t e = lists ? cudaFuncSetAttribute(k_hash_count<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)
                          : cudaFuncSetAttribute(k_hash_count<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  if (lists) k_hash_count<true><<<fd.n_segs, kHashThreads, sm, st>>>(sd, fd);
  else k_hash_count<false><<<fd.n_segs, kHashThreads, sm, st>>>(sd, fd);
  return cudaGetLastError();
}

cudaError_t launch_plan(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  k_plan_prep<<<1, kPlanThreads, 0, st>>>(sd, fd);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int wpb = kPlanRowsThreads / 32;
  k_plan_rows<<<(sd.P + wpb - 1) / wpb, kPlanRowsThreads, 0, st>>>(sd, fd);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (sd.n_str > 0) {
    const int n = sd.n_str * sd.P;
    k_plan_bytes<<<(n + wpb - 1) / wpb, kPlanRowsThreads, 0, st>>>(sd, fd);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  k_plan_scan<<<1, kPlanThreads, 0, st>>>(sd, fd);
  return cudaGetLastError();
}

cudaError_t launch_nest_prep(const NestJob* jobs, uint32_t n_jobs, int32_t* err, cudaStream_t st) {
  if (n_jobs == 0) return cudaSuccess;
  k_nest_prep<<<n_jobs < 1216u ? n_jobs : 1216u, 256, 0, st>>>(jobs, n_jobs, err);
  return cudaGetLastError();
}

cudaError_t launch_gather(const HostCopy* jobs, uint32_t n_jobs, cudaStream_t st) {
  if (n_jobs == 0) return cudaSuccess;
  // two CTAs per SM stride over the buffers: enough loads in flight to fill the host link
  // while leaving the SMs to the device pass that runs concurrently
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  }
  const uint32_t grid = n_jobs < (uint32_t)(2 * sms) ? n_jobs : (uint32_t)(2 * sms);
  k_gather<<<grid, 256, 0, st>>>(jobs, n_jobs);
  return cudaGetLastError();
}

size_t scatter_smem_bytes() {
  const int T = kTileRows;
  return kSlots * kStageSlot + kCharRegion + 4 * sizeof(uint16_t) * T +
         sizeof(uint16_t) * T + sizeof(uint32_t) * (T + 1) + 2 * sizeof(uint32_t) * T +
         sizeof(uint16_t) * kW * 256 + 3 * sizeof(uint32_t) * T;
}

cudaError_t launch_scatter(const SchemaDesc& sd, const FlushDesc& fd, cudaStream_t st) {
  const size_t sm = scatter_smem_bytes();
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  if (sd.list_mask) k_scatter<true><<<fd.n_tiles, kScatterBlock, sm, st>>>(sd, fd);
  else k_scatter<false><<<fd.n_tiles, kScatterBlock, sm, st>>>(sd, fd);
  return cudaGetLastError();
}

int max_str_columns() { return kMaxStrPlan; }

}  // namespace gz
