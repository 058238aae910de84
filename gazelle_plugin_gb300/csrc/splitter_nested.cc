// Nested columns of the splitter: list / large_list / map / struct of any depth (the reference's
// list_array_idx_ columns, split by SplitListArray / AppendList through the Arrow builders'
// AppendArraySlice, native-sql-engine/cpp/src/shuffle/splitter.cc:1322-1344, and finished by
// CacheRecordBatch, :532-545).
//
// The builders append, per row, one slice of every node of the column's type tree: a list / map
// entry's elements when it is valid (none when it is null), a struct's children for every entry,
// a string's bytes when it is valid, fixed-width values and bool bits always.  So a top-level row
// selects one contiguous range of every node's entries, and a partition's output at a node is the
// concatenation of its rows' ranges in row order - what the device's list-like columns (a row:
// a range of elements, copied to its partition in a stable order) already produce.  Each node
// becomes such a column ("stream", see splitter.h), Stop rebuilds the tree from them.
//
// One case is refused: a null list, map or string entry below a list or map that holds elements
// (its builder drops them, which would split the range).  Arrow writers give null entries empty
// ranges; k_nest_prep reports the case (GZ_NOT_IMPLEMENTED).
#include <string.h>

#include <algorithm>
#include <map>

#include "gz_kernels.h"
#include "split_util.h"
#include "splitter.h"

namespace gz {

namespace {

bool ListLike(int t) { return t == GZ_TYPE_LIST || t == GZ_TYPE_LARGE_LIST || t == GZ_TYPE_MAP; }
// offset bytes of a node with offsets
int NodeOffW(int t) { return t == GZ_TYPE_LARGE_LIST ? 8 : IsBinary(t) ? OffW(t) : 4; }

}  // namespace

int NestedBufferCount(const Field& f) {
  if (f.type == GZ_TYPE_LIST && !f.nested()) return 4;  // [validity, offsets, element validity, values]
  int n = f.type == GZ_TYPE_STRUCT ? 1 : ListLike(f.type) ? 2 : IsBinary(f.type) ? 3 : 2;
  for (const Field& c : f.children) n += NestedBufferCount(c);
  return n;
}

// Pre-order nodes with their buffers (MakeArrayData's order: a node's own buffers, then its
// children's); a list in the simple form gets its element leaf as a child node.
void Splitter::PlanNode(NestPlan& np, const Field& f, int parent, int* buf) {
  const int idx = (int)np.nodes.size();
  np.nodes.push_back(NestNode());
  np.nodes[idx].type = f.type;
  np.nodes[idx].width = ByteWidth(f.type);
  np.nodes[idx].parent = parent;
  np.nodes[idx].buf = *buf;
  *buf += f.type == GZ_TYPE_STRUCT ? 1 : ListLike(f.type) ? 2 : IsBinary(f.type) ? 3 : 2;
  if (parent >= 0) np.nodes[parent].kids.push_back(idx);
  if (f.type == GZ_TYPE_LIST && !f.nested()) {
    Field e;
    e.type = f.elem;
    e.nullable = f.elem_nullable;
    e.name = f.elem_name;
    PlanNode(np, e, idx, buf);
    return;
  }
  for (const Field& c : f.children) PlanNode(np, c, idx, buf);
}

namespace {

// Where each node's entries come from: `ident` (the rows), or the chain of list / map nodes
// whose offsets lead to them; `mask`: the outermost list / map whose entries are rows (its null
// rows select nothing below it).
void AssignRanges(std::vector<Splitter::NestNode>& nodes, int i, bool ident, bool inner, int mask,
                  const std::vector<int>& chain) {
  nodes[i].ident = ident;
  nodes[i].inner = inner;
  nodes[i].mask = mask;
  nodes[i].chain = chain;
  const std::vector<int> kids = nodes[i].kids;
  if (nodes[i].type == GZ_TYPE_STRUCT) {
    for (int k : kids) AssignRanges(nodes, k, ident, inner, mask, chain);
  } else if (ListLike(nodes[i].type)) {
    std::vector<int> c2 = chain;
    c2.push_back(i);
    for (int k : kids) AssignRanges(nodes, k, false, true, ident ? i : mask, c2);
  }
}

int PayloadOf(const Splitter::NestNode& nd) {
  if (nd.type == GZ_TYPE_STRUCT) return Splitter::PAY_NONE;
  if (nd.type == GZ_TYPE_BOOL) return Splitter::PAY_BITS;
  if (ListLike(nd.type) || IsBinary(nd.type)) return Splitter::PAY_LENGTHS;
  return Splitter::PAY_VALUES;
}

}  // namespace

Status Splitter::PlanNested() {
  for (size_t i = 0; i < fields_.size(); i++) {
    if ((int)i == pid_field_ || !fields_[i].nested()) continue;
    NestPlan np;
    np.field = (int)i;
    int buf = 0;
    PlanNode(np, fields_[i], -1, &buf);
    for (const NestNode& nd : np.nodes) {
      const bool ok = nd.type == GZ_TYPE_STRUCT ? !nd.kids.empty()
                      : ListLike(nd.type)      ? nd.kids.size() == 1
                      : IsBinary(nd.type) || nd.type == GZ_TYPE_BOOL || nd.width > 0;
      if (!ok) return Status::Error(GZ_NOT_IMPLEMENTED, "nested field type not implemented in ColumnarShuffle");
      if (nd.type == GZ_TYPE_MAP) {
        const NestNode& e = np.nodes[nd.kids[0]];
        if (e.type != GZ_TYPE_STRUCT || e.kids.size() != 2)
          return Status::Error(GZ_INVALID, "Map array child array should have two fields");
      }
    }
    AssignRanges(np.nodes, 0, true, false, -1, {});
    for (const NestNode& nd : np.nodes)
      if (nd.chain.size() + 1 > (size_t)kMaxNestChain)
        return Status::Error(GZ_NOT_IMPLEMENTED, "nested column deeper than 5 lists / maps");
    // a top-level list or map shares its child's stream (its 32-bit row offsets are that stream's);
    // a large_list's entries get a stream of their own (their lengths rebuild its 64-bit offsets)
    np.root_list = np.nodes[0].type == GZ_TYPE_LIST || np.nodes[0].type == GZ_TYPE_MAP;
    nest_.push_back(std::move(np));
  }
  for (size_t pi = 0; pi < nest_.size(); pi++) {
    NestPlan& np = nest_[pi];
    auto add = [&](int node, bool chars, int payload) {
      const int a = (int)array_idx_.size();
      array_idx_.push_back(np.field);
      Stream sm;
      sm.plan = (int)pi;
      sm.node = node;
      sm.chars = chars;
      sm.payload = payload;
      sm.slot = n_slots_++;
      streams_.push_back(sm);
      return a;
    };
    for (int i = 0; i < (int)np.nodes.size(); i++) {
      NestNode& nd = np.nodes[i];
      if (i == 0 && np.root_list) continue;  // shares its child's stream
      const bool under_root = np.root_list && nd.parent == 0;
      const bool map_entries = nd.parent >= 0 && np.nodes[nd.parent].type == GZ_TYPE_MAP;
      if (map_entries) {
        // the entries struct of a map is all valid and carries nothing: a stream only where the
        // map is the root (its rows' ranges and validity)
        if (under_root) np.nodes[0].stream = nd.stream = add(i, false, PAY_NONE);
      } else {
        nd.stream = add(i, false, PayloadOf(nd));
        if (under_root) np.nodes[0].stream = nd.stream;
      }
      if (IsBinary(nd.type)) nd.chars = add(i, true, PAY_VALUES);
    }
  }
  return Status::OK();
}

Status Splitter::EnsureIota(uint32_t rows) {
  if ((uint64_t)rows + 1 <= iota_cap_) return Status::OK();
  const uint32_t cap = std::max<uint32_t>({rows + 1, 65537u, iota_cap_ * 2});
  // (64 entries of slack: a staged slice rounded up to 16 bytes stays inside the allocation)
  std::vector<int32_t> h((size_t)cap + 64);
  for (size_t i = 0; i < h.size(); i++) h[i] = (int32_t)i;
  int32_t* d = nullptr;
  Status st = Cuda(cudaMalloc(reinterpret_cast<void**>(&d), h.size() * 4), "cudaMalloc(iota)");
  if (!st.ok()) return st;
  st = Cuda(cudaMemcpy(d, h.data(), h.size() * 4, cudaMemcpyHostToDevice), "H2D iota");
  if (!st.ok()) {
    cudaFree(d);
    return st;
  }
  if (d_iota_) old_iota_.push_back(d_iota_);  // passes in flight may still read it
  d_iota_ = d;
  iota_cap_ = cap;
  return Status::OK();
}

// The streams' ColPtr slots of one batch, their derived arrays (queued for the pass) and the
// bytes their outputs may need.  `dptr`: device address of every input buffer (nullptr: empty).
Status Splitter::StageNested(uint32_t nr, const int64_t* addrs, const int64_t* sizes, const uint8_t* const* dptr,
                             ColPtr* cols, bool host_in) {
  if (nest_.empty()) return Status::OK();
  Status st = EnsureIota(nr);
  if (!st.ok()) return st;
  const uint32_t b = (uint32_t)pending_.size();
  auto size_of = [&](int buf) -> int64_t { return addrs[buf] != 0 ? std::max<int64_t>(sizes[buf], 0) : 0; };
  for (const NestPlan& np : nest_) {
    const int nn = (int)np.nodes.size();
    // entries of every node: the rows where they are rows, else as MakeArrayData reads them
    std::vector<int64_t> m(nn, 0);
    for (int i = nn - 1; i >= 0; i--) {
      const NestNode& nd = np.nodes[i];
      if (nd.ident) {
        m[i] = nr;
      } else if (ListLike(nd.type) || IsBinary(nd.type)) {
        m[i] = std::max<int64_t>(size_of(nd.buf + 1) / NodeOffW(nd.type) - 1, 0);
      } else if (nd.type == GZ_TYPE_BOOL) {
        m[i] = size_of(nd.buf + 1) * 8;
      } else if (nd.type == GZ_TYPE_STRUCT) {
        m[i] = INT64_MAX;
        for (int k : nd.kids) m[i] = std::min(m[i], m[k]);
      } else {
        m[i] = size_of(nd.buf + 1) / nd.width;
      }
    }
    // buffers the row-level nodes must hold for nr rows
    for (int i = 0; i < nn; i++) {
      const NestNode& nd = np.nodes[i];
      const bool entries = nd.parent >= 0 && np.nodes[nd.parent].type == GZ_TYPE_MAP;
      const int64_t vb = size_of(nd.buf);
      if (vb > 0 && !entries && vb < BytesForBits(m[i])) return Status::Error(GZ_INVALID, "validity buffer too small");
      if (!nd.ident) continue;
      if (ListLike(nd.type) || IsBinary(nd.type)) {
        if (size_of(nd.buf + 1) < (int64_t)(nr + 1) * NodeOffW(nd.type))
          return Status::Error(GZ_INVALID, "offsets buffer too small");
      } else if (nd.type == GZ_TYPE_BOOL || nd.width > 0) {
        if (size_of(nd.buf + 1) < (nd.width ? (int64_t)nr * nd.width : BytesForBits(nr)))
          return Status::Error(GZ_INVALID, "value buffer too small");
      }
    }
    if (!host_in) {
      for (int i = 0; i < nn; i++) {
        const NestNode& nd = np.nodes[i];
        const int ow = NodeOffW(nd.type);
        if ((ListLike(nd.type) || IsBinary(nd.type)) && reinterpret_cast<uintptr_t>(dptr[nd.buf + 1]) % ow)
          return Status::Error(GZ_INVALID, "device offsets buffer must be aligned to its offset width");
        if (nd.width > 0 && reinterpret_cast<uintptr_t>(dptr[nd.buf + 1]) % nd.width)
          return Status::Error(GZ_INVALID, "device value buffer is not aligned to its width");
      }
    }
    // composed row ranges, shared by the streams with the same chain
    std::map<std::vector<int>, int> composed;  // chain -> pending_derived_ index
    // one row range end of a chain, read on the host (host inputs): entries [lo, hi) of the rows
    auto host_end = [&](const std::vector<int>& chain, int64_t r, int64_t* out) -> bool {
      int64_t x = r;
      for (int c : chain) {
        const NestNode& cn = np.nodes[c];
        const int ow = NodeOffW(cn.type);
        if (x < 0 || x >= size_of(cn.buf + 1) / ow) return false;
        x = OffAt(reinterpret_cast<const uint8_t*>(addrs[cn.buf + 1]), ow, (size_t)x);
      }
      *out = x;
      return x >= 0 && x <= INT32_MAX;
    };
    for (size_t si = 0; si < streams_.size(); si++) {
      const Stream& sm = streams_[si];
      if (&nest_[sm.plan] != &np) continue;
      const int a = first_stream_ + (int)si;
      const NestNode& nd = np.nodes[sm.node];
      std::vector<int> chain = nd.chain;
      if (sm.chars) chain.push_back(sm.node);
      const int maskn = sm.chars ? (nd.ident ? sm.node : nd.mask) : nd.mask;
      ColPtr cp{nullptr, nullptr, nullptr, 0, nullptr};
      if (maskn >= 0) cp.validity = dptr[np.nodes[maskn].buf];
      const bool entries = nd.parent >= 0 && np.nodes[nd.parent].type == GZ_TYPE_MAP;
      if (!sm.chars && !entries) cp.child_validity = dptr[nd.buf];
      // row ranges
      if (chain.empty()) {
        cp.offsets = d_iota_;
      } else if (chain.size() == 1 && NodeOffW(np.nodes[chain[0]].type) == 4) {
        cp.offsets = reinterpret_cast<const int32_t*>(dptr[np.nodes[chain[0]].buf + 1]);
        if (cp.offsets == nullptr) return Status::Error(GZ_INVALID, "offsets buffer too small");
      } else {
        auto it = composed.find(chain);
        if (it == composed.end()) {
          PendingDerived pd;
          memset(&pd.job, 0, sizeof(pd.job));
          pd.batch = b;
          pd.slot = sm.slot;
          pd.values = false;
          pd.same_as = -1;
          pd.job.kind = 0;
          pd.job.n = nr + 1;
          pd.job.depth = (uint32_t)chain.size();
          for (size_t d = 0; d < chain.size(); d++) {
            const NestNode& cn = np.nodes[chain[d]];
            const int ow = NodeOffW(cn.type);
            pd.job.off[d] = dptr[cn.buf + 1];
            pd.job.lim[d] = (uint64_t)(size_of(cn.buf + 1) / ow);
            pd.job.wide[d] = ow == 8;
          }
          pd.bytes = (size_t)(nr + 1) * 4;
          composed[chain] = (int)pending_derived_.size();
          pending_derived_.push_back(pd);
        } else {  // the same array, pointed at from this slot too
          PendingDerived pd = pending_derived_[it->second];
          pd.slot = sm.slot;
          pd.same_as = it->second;
          pending_derived_.push_back(pd);
        }
      }
      // payload
      const int k = a - fixed_cnt_;
      const int sh = sd_.arr_shift[a];
      int64_t cap_elems = m[sm.node];
      if (sm.chars) {
        cp.values = dptr[nd.buf + 2];
        cp.values_bytes = (uint64_t)size_of(nd.buf + 2);
        cap_elems = size_of(nd.buf + 2);
      } else if (sm.payload == PAY_VALUES || sm.payload == PAY_BITS) {
        cp.values = dptr[nd.buf + 1];
        cp.values_bytes = (uint64_t)size_of(nd.buf + 1);
      } else if (sm.payload == PAY_LENGTHS && m[sm.node] > 0) {
        PendingDerived pd;
        memset(&pd.job, 0, sizeof(pd.job));
        pd.batch = b;
        pd.slot = sm.slot;
        pd.values = true;
        pd.same_as = -1;
        pd.job.kind = 1;
        pd.job.n = (uint32_t)m[sm.node];
        pd.job.depth = 1;
        pd.job.inner = nd.inner ? 1 : 0;
        const int ow = NodeOffW(nd.type);
        pd.job.off[0] = dptr[nd.buf + 1];
        pd.job.lim[0] = (uint64_t)(size_of(nd.buf + 1) / ow);
        pd.job.wide[0] = ow == 8;
        pd.job.validity = entries ? nullptr : dptr[nd.buf];
        pd.job.lim[1] = (uint64_t)size_of(nd.buf) * 8;
        pd.bytes = (size_t)m[sm.node] * 4;
        pending_derived_.push_back(pd);
        cp.values_bytes = (uint64_t)m[sm.node] * 4;
      } else if (sm.payload == PAY_NONE) {
        cp.values_bytes = (uint64_t)BytesForBits(m[sm.node]);
      }
      if (m[sm.node] > INT32_MAX / 16 || cp.values_bytes > (uint64_t)INT32_MAX)
        return Status::Error(GZ_NOT_IMPLEMENTED, "a nested column batch with more than 2^31 - 1 element bytes");
      if (cp.values == nullptr) cp.values = reinterpret_cast<const uint8_t*>(d_iota_);  // nothing read
      // what the pass output may need for this batch
      uint64_t elems = (uint64_t)std::max<int64_t>(cap_elems, 0);
      if (host_in) {
        int64_t lo = 0, hi = nr;
        if (!chain.empty() && (!host_end(chain, 0, &lo) || !host_end(chain, nr, &hi) || hi < lo))
          return Status::Error(GZ_INVALID, "nested offsets exceed their children");
        elems = (uint64_t)(hi - lo);
      }
      char_scratch_[k] = (sm.payload == PAY_BITS || sm.payload == PAY_NONE) && !sm.chars ? elems : elems << sh;
      cols[sm.slot] = cp;
    }
  }
  return Status::OK();
}

// ---------------------------------------------------------------------------------------
// Stop: one nested field of one record batch, as its builders finish it - the nodes in pre-order,
// each with [validity (only with a null, zero-padded), offsets (list / map / binary, from 0),
// values (fixed width, bool bits, binary bytes)].
void Splitter::BuildNested(int p, const Segment& s, const NestPlan& np, int i, std::vector<FieldNodeMeta>* nodes,
                           std::vector<ChunkedBuffer>* bufs, std::vector<std::vector<uint8_t>>* temps,
                           bool device_view, int64_t* raw) const {
  const int P = P_;
  const int nstr = n_str_;
  const NestNode& nd = np.nodes[i];
  auto body_base = [&](const FlushRec& f, bool* dev) -> const uint8_t* {
    *dev = device_view;
    return device_view && !f.on_host ? f.d_out : f.h_out;
  };
  auto bit_base = [&](const FlushRec& f, size_t off) -> const uint8_t* {
    return f.on_host ? f.h_out + off : f.h_bits + (off - f.bits_begin);
  };
  auto new_temp = [&](size_t bytes, uint8_t fill) -> uint8_t* {
    temps->emplace_back(bytes, fill);
    return temps->back().data();
  };

  if (i == 0 && np.root_list) {
    // the top-level list / map: the stream's rows - its validity and offsets
    const int a = nd.stream;
    const uint32_t n = s.rows;
    int64_t nulls = 0;
    ChunkedBuffer vb;
    {
      uint8_t* bits = new_temp((size_t)BytesForBits(n), 0xff);
      uint64_t drow = 0;
      bool any = false;
      for (const Piece& pc : s.pieces) {
        const FlushRec& f = flushes_[pc.flush];
        const uint32_t len = pc.frow1 - pc.frow0;
        if (f.off_valid[a] != SIZE_MAX) {
          CopyBits(bit_base(f, f.off_valid[a]), (uint64_t)f.vstart(P)[p] + pc.vpos0, bits, drow, len);
          any = true;
        }
        drow += len;
      }
      if (any && (nulls = CountZeros(bits, n)) > 0) {
        if (n & 7) bits[n >> 3] &= (uint8_t)((1u << (n & 7)) - 1);
        vb.push_back(Chunk{bits, BytesForBits(n)});
      }
    }
    static const uint8_t kZero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    ChunkedBuffer ob;
    const int ow = 4;
    ob.push_back(Chunk{kZero8, 4});
    for (const Piece& pc : s.pieces) {
      const FlushRec& f = flushes_[pc.flush];
      bool dev;
      const uint8_t* fb = body_base(f, &dev);
      ob.push_back(Chunk{fb + f.off_values[a] + ((size_t)f.pstart(P)[p] + pc.frow0) * 4,
                         (int64_t)(pc.frow1 - pc.frow0) * 4, dev});
    }
    nodes->push_back(FieldNodeMeta{n, nulls});
    bufs->push_back(vb);
    bufs->push_back(ob);
    *raw += (nulls > 0 ? BytesForBits(n) : 0) + (int64_t)(n + 1) * ow;  // batch_nbytes: own buffers
    for (int k : nd.kids) BuildNested(p, s, np, k, nodes, bufs, temps, device_view, raw);
    return;
  }

  if (nd.stream < 0) {
    // a map's entries struct: all valid, as many entries as keys
    const NestNode& key = np.nodes[nd.kids[0]];
    const int ka = key.stream;
    const int kk = sd_.arr_str[ka], ksh = sd_.arr_shift[ka];
    uint64_t elems = 0;
    for (const Piece& pc : s.pieces) elems += (pc.fb1[kk] - pc.fb0[kk]) >> ksh;
    nodes->push_back(FieldNodeMeta{(int64_t)elems, 0});
    bufs->push_back(ChunkedBuffer{});
    for (int k : nd.kids) BuildNested(p, s, np, k, nodes, bufs, temps, device_view, raw);
    return;
  }

  const int a = nd.stream;
  const int k = sd_.arr_str[a];
  const int sh = sd_.arr_shift[a];
  uint64_t elems = 0;
  for (const Piece& pc : s.pieces) elems += (pc.fb1[k] - pc.fb0[k]) >> sh;
  // validity: the stream's element validity
  int64_t nulls = 0;
  ChunkedBuffer vb;
  {
    uint8_t* ev = new_temp((size_t)BytesForBits((int64_t)elems), 0);
    uint64_t at = 0;
    for (const Piece& pc : s.pieces) {
      const FlushRec& f = flushes_[pc.flush];
      const uint64_t cb = (uint64_t)f.cstart(P, nstr)[(size_t)k * P + p] + pc.fb0[k];
      const uint64_t m = (pc.fb1[k] - pc.fb0[k]) >> sh;
      if (f.off_cvalid[a] != SIZE_MAX) CopyBits(bit_base(f, f.off_cvalid[a]), cb >> sh, ev, at, m);
      else
        for (uint64_t x = at; x < at + m; x++) ev[x >> 3] |= (uint8_t)(1u << (x & 7));
      at += m;
    }
    nulls = CountZeros(ev, (int64_t)elems);
    if (nulls > 0) vb.push_back(Chunk{ev, BytesForBits((int64_t)elems)});
  }
  nodes->push_back(FieldNodeMeta{(int64_t)elems, nulls});
  bufs->push_back(vb);
  if (i == 0)  // batch_nbytes: a top-level struct's validity, a large_list's validity and offsets
    *raw += (nulls > 0 ? BytesForBits((int64_t)elems) : 0) +
            (ListLike(nd.type) ? (int64_t)(elems + 1) * NodeOffW(nd.type) : 0);

  const int payload = streams_[a - first_stream_].payload;
  if (payload == PAY_VALUES) {
    ChunkedBuffer vals;
    for (const Piece& pc : s.pieces) {
      if (pc.fb1[k] == pc.fb0[k]) continue;
      const FlushRec& f = flushes_[pc.flush];
      bool dev;
      const uint8_t* fb = body_base(f, &dev);
      const size_t cb = (size_t)f.cstart(P, nstr)[(size_t)k * P + p] + pc.fb0[k];
      vals.push_back(Chunk{fb + f.off_chars[a] + cb, (int64_t)(pc.fb1[k] - pc.fb0[k]), dev});
    }
    bufs->push_back(vals);
  } else if (payload == PAY_BITS) {
    uint8_t* bv = new_temp((size_t)BytesForBits((int64_t)elems), 0);
    uint64_t at = 0;
    for (const Piece& pc : s.pieces) {
      const FlushRec& f = flushes_[pc.flush];
      const uint64_t cb = (uint64_t)f.cstart(P, nstr)[(size_t)k * P + p] + pc.fb0[k];
      const uint64_t m = pc.fb1[k] - pc.fb0[k];
      CopyBits(bit_base(f, f.off_chars[a]), cb, bv, at, m);
      at += m;
    }
    bufs->push_back(ChunkedBuffer{Chunk{bv, BytesForBits((int64_t)elems)}});
  } else if (payload == PAY_LENGTHS) {
    // offsets from 0: a running sum of the entries' lengths
    const int ow = NodeOffW(nd.type);
    uint8_t* ob = new_temp((size_t)(elems + 1) * ow, 0);
    int64_t run = 0;
    uint64_t at = 1;
    for (const Piece& pc : s.pieces) {
      const FlushRec& f = flushes_[pc.flush];
      const size_t cb = (size_t)f.cstart(P, nstr)[(size_t)k * P + p] + pc.fb0[k];
      const int32_t* len = reinterpret_cast<const int32_t*>(bit_base(f, f.off_chars[a]) + cb);
      const uint64_t m = (pc.fb1[k] - pc.fb0[k]) >> 2;
      for (uint64_t x = 0; x < m; x++, at++) {
        run += len[x];
        if (ow == 8) memcpy(ob + at * 8, &run, 8);
        else {
          const int32_t v = (int32_t)run;
          memcpy(ob + at * 4, &v, 4);
        }
      }
    }
    bufs->push_back(ChunkedBuffer{Chunk{ob, (int64_t)(elems + 1) * ow}});
    if (IsBinary(nd.type)) {  // the characters
      const int ca = nd.chars;
      const int ck = sd_.arr_str[ca];
      ChunkedBuffer chars;
      for (const Piece& pc : s.pieces) {
        if (pc.fb1[ck] == pc.fb0[ck]) continue;
        const FlushRec& f = flushes_[pc.flush];
        bool dev;
        const uint8_t* fb = body_base(f, &dev);
        const size_t cb = (size_t)f.cstart(P, nstr)[(size_t)ck * P + p] + pc.fb0[ck];
        chars.push_back(Chunk{fb + f.off_chars[ca] + cb, (int64_t)(pc.fb1[ck] - pc.fb0[ck]), dev});
      }
      bufs->push_back(chars);
    }
  }
  for (int kid : nd.kids) BuildNested(p, s, np, kid, nodes, bufs, temps, device_view, raw);
}

// ---------------------------------------------------------------------------------------
// CompressedSize: the body buffers Arrow's IPC writer takes for entries [off, off + len) of a
// nested node of the input batch (RecordBatchSerializer: a validity buffer only with a null,
// offsets from 0, children sliced to the entries' range).
void Splitter::NestedBodyBuffers(const NestPlan& np, int i, int64_t off, int64_t len, const int64_t* addrs,
                                 const int64_t* sizes, std::vector<std::pair<const uint8_t*, int64_t>>* out,
                                 std::vector<std::vector<uint8_t>>* temps) const {
  const NestNode& nd = np.nodes[i];
  const bool entries = nd.parent >= 0 && np.nodes[nd.parent].type == GZ_TYPE_MAP;
  const uint8_t* v = reinterpret_cast<const uint8_t*>(addrs[nd.buf]);
  const bool has_v = !entries && v != nullptr && sizes[nd.buf] > 0;
  bool any_null = false;
  if (has_v)
    for (int64_t r = off; r < off + len && !any_null; r++) any_null = !((v[r >> 3] >> (r & 7)) & 1);
  if (any_null) {
    temps->emplace_back((size_t)BytesForBits(len), 0);
    CopyBits(v, (uint64_t)off, temps->back().data(), 0, (uint64_t)len);
    out->push_back({temps->back().data(), BytesForBits(len)});
  } else {
    out->push_back({nullptr, 0});
  }
  if (nd.type == GZ_TYPE_STRUCT) {
    for (int k : nd.kids) NestedBodyBuffers(np, k, off, len, addrs, sizes, out, temps);
    return;
  }
  if (ListLike(nd.type) || IsBinary(nd.type)) {
    const int ow = NodeOffW(nd.type);
    const uint8_t* o = reinterpret_cast<const uint8_t*>(addrs[nd.buf + 1]);
    const int64_t lim = sizes[nd.buf + 1] / ow;
    auto at = [&](int64_t r) -> int64_t { return o != nullptr && r < lim ? OffAt(o, ow, (size_t)r) : 0; };
    const int64_t o0 = len > 0 ? at(off) : 0;
    temps->emplace_back((size_t)(len + 1) * ow, 0);
    uint8_t* z = temps->back().data();
    for (int64_t r = 0; r <= len && len > 0; r++) {
      const int64_t x = at(off + r) - o0;
      if (ow == 8) memcpy(z + r * 8, &x, 8);
      else {
        const int32_t y = (int32_t)x;
        memcpy(z + r * 4, &y, 4);
      }
    }
    out->push_back({z, (int64_t)(len + 1) * ow});
    const int64_t o1 = len > 0 ? at(off + len) : 0;
    if (IsBinary(nd.type)) {
      out->push_back({reinterpret_cast<const uint8_t*>(addrs[nd.buf + 2]) + o0, o1 - o0});
      return;
    }
    for (int k : nd.kids) NestedBodyBuffers(np, k, o0, o1 - o0, addrs, sizes, out, temps);
    return;
  }
  const uint8_t* vals = reinterpret_cast<const uint8_t*>(addrs[nd.buf + 1]);
  if (nd.type == GZ_TYPE_BOOL) {
    temps->emplace_back((size_t)BytesForBits(len), 0);
    if (vals) CopyBits(vals, (uint64_t)off, temps->back().data(), 0, (uint64_t)len);
    out->push_back({temps->back().data(), BytesForBits(len)});
  } else {
    out->push_back({vals + off * nd.width, len * nd.width});
  }
}

}  // namespace gz
