// Host-side leaf forest: refinement / coarsening of the leaf blocks, 2:1 balance across faces, edges
// and corners, and the mesh tables the kernels read (p4est's adapt + balance + the reference's
// orchard-key hashmap lookups, SolverGodunovMHD.cpp:263-319; p4est_balance with full connectivity).
//
// Leaves are keyed by (level, x, y, z) with x, y, z the block position at that level over a brick of
// bricks[0] x bricks[1] x bricks[2] trees. Block order is p4est's: trees x fastest, then the Morton
// order of the block's anchor at the finest level present.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/gmhd.h"

namespace
{
struct Key
{
  int32_t L, x, y, z;
};

inline uint64_t
pack(int L, int x, int y, int z)
{
  return ((uint64_t)(uint32_t)L << 57) | ((uint64_t)(uint32_t)x << 38) | ((uint64_t)(uint32_t)y << 19) |
         (uint64_t)(uint32_t)z;
}

inline Key
unpack(uint64_t k)
{
  return Key{(int)(k >> 57), (int)((k >> 38) & 0x7ffff), (int)((k >> 19) & 0x7ffff), (int)(k & 0x7ffff)};
}

// Open-addressing table of packed keys -> int32 (linear probing, Fibonacci hashing, backward-shift
// erase). The all-ones key never occurs (levels stop at 18), so it marks an empty slot.
class KeyTable
{
public:
  explicit KeyTable(size_t n = 0) { rehash(capacity_for(n)); }

  size_t
  size() const
  {
    return n_;
  }
  const int32_t *
  find(uint64_t k) const
  {
    for (size_t i = home(k);; i = (i + 1) & mask_)
    {
      if (slots_[i].key == k)
        return &slots_[i].val;
      if (slots_[i].key == EMPTY)
        return nullptr;
    }
  }
  bool
  contains(uint64_t k) const
  {
    return find(k) != nullptr;
  }
  // insert, or overwrite the value of a present key; true when the key was new
  bool
  put(uint64_t k, int32_t v = 0)
  {
    if (2 * (n_ + 1) > slots_.size())
      rehash(2 * slots_.size());
    size_t i = home(k);
    for (; slots_[i].key != EMPTY; i = (i + 1) & mask_)
      if (slots_[i].key == k)
      {
        slots_[i].val = v;
        return false;
      }
    slots_[i] = Slot{k, v};
    ++n_;
    return true;
  }
  bool
  erase(uint64_t k)
  {
    size_t i = home(k);
    for (; slots_[i].key != k; i = (i + 1) & mask_)
      if (slots_[i].key == EMPTY)
        return false;
    // shift the rest of the probe run back so that no lookup stops early at the hole
    for (size_t j = (i + 1) & mask_; slots_[j].key != EMPTY; j = (j + 1) & mask_)
    {
      const size_t h = home(slots_[j].key);
      const bool   stays = (i <= j) ? (i < h && h <= j) : (i < h || h <= j);
      if (stays)
        continue;
      slots_[i] = slots_[j];
      i = j;
    }
    slots_[i].key = EMPTY;
    --n_;
    return true;
  }
  template <typename F>
  void
  for_each(F && f) const
  {
    for (const Slot & sl : slots_)
      if (sl.key != EMPTY)
        f(sl.key, sl.val);
  }
  std::vector<uint64_t>
  keys() const
  {
    std::vector<uint64_t> out;
    out.reserve(n_);
    for_each([&](uint64_t k, int32_t) { out.push_back(k); });
    return out;
  }

private:
  static constexpr uint64_t EMPTY = ~0ull;
  struct Slot
  {
    uint64_t key; // key and value side by side: one cache line per probe
    int32_t  val;
  };
  std::vector<Slot> slots_;
  size_t            mask_ = 0, n_ = 0;
  int               shift_ = 60;

  static size_t
  capacity_for(size_t n)
  {
    size_t c = 16;
    while (c < 2 * n + 2)
      c <<= 1;
    return c;
  }
  size_t
  home(uint64_t k) const
  {
    return (size_t)((k * 0x9E3779B97F4A7C15ull) >> shift_);
  }
  void
  rehash(size_t cap)
  {
    std::vector<Slot> old;
    old.swap(slots_);
    slots_.assign(cap, Slot{EMPTY, 0});
    mask_ = cap - 1;
    shift_ = 64;
    for (size_t c = cap; c > 1; c >>= 1)
      --shift_;
    n_ = 0;
    for (const Slot & sl : old)
      if (sl.key != EMPTY)
        put(sl.key, sl.val);
  }
};

struct Forest
{
  int dim = 3, bricks[3] = {1, 1, 1}, per[3] = {1, 1, 1}, base = 0;
  int offs[26][3];
  int noffs = 0;

  void
  init()
  {
    noffs = 0;
    for (int oz = (dim == 3 ? -1 : 0); oz <= (dim == 3 ? 1 : 0); ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox)
          if (ox || oy || oz)
          {
            offs[noffs][0] = ox;
            offs[noffs][1] = oy;
            offs[noffs][2] = oz;
            ++noffs;
          }
  }
  int
  ext(int L, int d) const
  {
    return d < dim ? bricks[d] << L : 1;
  }
  // c mod e for the coordinates of neighbour regions (at most one block width outside [0, e))
  static int
  periodic(int c, int e)
  {
    if (c < 0)
      c += e;
    else if (c >= e)
      c -= e;
    return (c >= 0 && c < e) ? c : ((c % e) + e) % e;
  }
  // wrap c (level L) on periodic axes; false when outside a non-periodic border
  bool
  wrap(int L, int * c) const
  {
    for (int d = 0; d < 3; ++d)
    {
      const int e = ext(L, d);
      if (per[d])
        c[d] = periodic(c[d], e);
      else if (c[d] < 0 || c[d] >= e)
        return false;
    }
    return true;
  }
  int
  nkids() const
  {
    return 1 << dim;
  }
  // leaves of `leaves` two levels below coarsened parent p and next to it: the only old leaves that can
  // now be out of balance (before the coarsening they touched p's children)
  void
  fine_neighbours_of(const KeyTable & leaves, uint64_t p, std::vector<uint64_t> & out) const
  {
    const Key k = unpack(p);
    const int n2 = dim == 3 ? 4 : 1; // grandchildren per axis: 4 in x and y, 4 or 1 in z
    for (int o = 0; o < noffs; ++o)
    {
      int r[3] = {k.x + offs[o][0], k.y + offs[o][1], k.z + offs[o][2]};
      if (!wrap(k.L, r))
        continue;
      for (int gz = 0; gz < n2; ++gz)
        for (int gy = 0; gy < 4; ++gy)
          for (int gx = 0; gx < 4; ++gx)
          {
            const uint64_t g = pack(k.L + 2, 4 * r[0] + gx, 4 * r[1] + gy, dim == 3 ? 4 * r[2] + gz : 0);
            if (leaves.contains(g))
              out.push_back(g);
          }
    }
  }
  uint64_t
  kid(const Key & k, int c) const
  {
    return pack(k.L + 1, 2 * k.x + (c & 1), 2 * k.y + ((c >> 1) & 1), 2 * k.z + ((c >> 2) & 1));
  }

  // refine leaves until every leaf's face/edge/corner neighbours are within one level. The work list
  // starts from `seeds` when given (the leaves that can break the balance of an already balanced
  // set), else from every leaf; the result (the coarsest balanced refinement) does not depend on it.
  void
  balance(KeyTable & leaves, const std::vector<uint64_t> * seeds = nullptr) const
  {
    std::vector<uint64_t> work = seeds ? *seeds : leaves.keys();
    while (!work.empty())
    {
      const uint64_t kk = work.back();
      work.pop_back();
      if (!leaves.contains(kk))
        continue;
      const Key k = unpack(kk);
      if (k.L - 2 < base)
        continue;
      for (int o = 0; o < noffs; ++o)
      {
        int r[3] = {k.x + offs[o][0], k.y + offs[o][1], k.z + offs[o][2]};
        if (!wrap(k.L, r))
          continue;
        // a leaf at L or L-1 covering r rules out a coarser one
        if (leaves.contains(pack(k.L, r[0], r[1], r[2])) || leaves.contains(pack(k.L - 1, r[0] >> 1, r[1] >> 1, r[2] >> 1)))
          continue;
        for (int lv = k.L - 2; lv >= base; --lv)
        {
          const int      sh = k.L - lv;
          const uint64_t anc = pack(lv, r[0] >> sh, r[1] >> sh, r[2] >> sh);
          if (leaves.erase(anc))
          {
            const Key a = unpack(anc);
            for (int c = 0; c < nkids(); ++c)
            {
              leaves.put(kid(a, c));
              work.push_back(kid(a, c));
            }
            work.push_back(kk);
            break;
          }
        }
      }
    }
  }
};

} // namespace

struct gmhd_forest
{
  int                   dim = 3, bx = 0, by = 0, bz = 0;
  int                   n_owned = 0, n_blocks = 0;
  bool                  has_fine = false;
  std::vector<int32_t>  level, coord, neighbor, out_src, out_normal, remap;
  std::vector<int64_t>  fine_at; // entries of the [n_blocks][27][8] children table that are not -1 ...
  std::vector<int32_t>  fine_id; // ... and their values
  std::vector<Key>      owned;
};

namespace
{
// fn(t, lo, hi) over [0, n) in contiguous ranges, one per host thread (up to 16; serial below 4,096
// items); range t precedes range t + 1, so results gathered per range keep the serial order
template <class F>
int
for_ranges(int n, F fn)
{
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int      nt = n < 4096 ? 1 : (int)std::min<unsigned>(hw, (unsigned)(n / 1024));
  if (nt <= 1)
  {
    fn(0, 0, n);
    return 1;
  }
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  for (int t = 1; t < nt; ++t)
    th.emplace_back([&, t] { fn(t, (int)((int64_t)t * n / nt), (int)((int64_t)(t + 1) * n / nt)); });
  fn(0, 0, (int)((int64_t)n / nt));
  for (std::thread & x : th)
    x.join();
  return nt;
}

// mesh tables of a balanced leaf set
// every third bit of v (v < 2^21): the usual "part 1 by 2" interleave by shifts and masks
inline uint64_t
spread3(uint64_t v)
{
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

void
build(const Forest & f, const KeyTable & leaves, gmhd_forest & out)
{
  const std::vector<uint64_t> keys = leaves.keys();
  int                         max_level = 0;
  for (uint64_t k : keys)
    max_level = std::max(max_level, unpack(k).L);
  // p4est order: tree (bricks x fastest), then the Morton code of the leaf's anchor at max_level
  // (leaves of a leaf set never share an anchor)
  struct Ord
  {
    uint64_t tree, morton;
    uint64_t key;
  };
  std::vector<Ord> ord;
  ord.reserve(keys.size());
  for (uint64_t kk : keys)
  {
    const Key k = unpack(kk);
    const int t[3] = {k.x >> k.L, k.y >> k.L, k.z >> k.L};
    const uint64_t tid = (uint64_t)t[0] + (uint64_t)f.bricks[0] * ((uint64_t)t[1] + (uint64_t)f.bricks[1] * t[2]);
    const int      sh = max_level - k.L;
    const uint64_t m = spread3((uint64_t)(k.x - (t[0] << k.L)) << sh) |
                       spread3((uint64_t)(k.y - (t[1] << k.L)) << sh) << 1 |
                       spread3((uint64_t)(k.z - (t[2] << k.L)) << sh) << 2;
    ord.push_back(Ord{tid, m, kk});
  }
  const uint64_t ntrees = (uint64_t)f.bricks[0] * f.bricks[1] * f.bricks[2];
  if (3 * max_level + 64 - __builtin_clzll(ntrees | 1) <= 64)
  {
    // one 64-bit sort key: tree id above the Morton bits; least-significant-digit radix sort over
    // the bits in use, 11 bits per pass (keys are distinct, so stability only orders the passes)
    uint64_t top = 0;
    for (Ord & o : ord)
    {
      o.morton |= o.tree << (3 * max_level);
      top |= o.morton;
    }
    const int        nbits = top ? 64 - __builtin_clzll(top) : 1;
    std::vector<Ord> tmp(ord.size());
    std::vector<uint32_t> cnt(1u << 11);
    for (int shift = 0; shift < nbits; shift += 11)
    {
      std::fill(cnt.begin(), cnt.end(), 0u);
      for (const Ord & o : ord)
        ++cnt[(o.morton >> shift) & 0x7ff];
      uint32_t sum = 0;
      for (uint32_t & c : cnt)
      {
        const uint32_t c0 = c;
        c = sum;
        sum += c0;
      }
      for (const Ord & o : ord)
        tmp[cnt[(o.morton >> shift) & 0x7ff]++] = o;
      ord.swap(tmp);
    }
  }
  else
    std::sort(ord.begin(), ord.end(), [](const Ord & p, const Ord & q) {
      return p.tree != q.tree ? p.tree < q.tree : p.morton < q.morton;
    });
  KeyTable ids(ord.size());
  out.owned.clear();
  out.owned.reserve(ord.size());
  for (size_t n = 0; n < ord.size(); ++n)
  {
    ids.put(ord[n].key, (int32_t)n);
    out.owned.push_back(unpack(ord[n].key));
  }
  const int n_owned = (int)ord.size();
  // outside blocks at the level of the block they serve, sourced from the same-level inside block
  KeyTable         out_ids;
  std::vector<Key> out_keys;
  out.out_src.clear();
  out.out_normal.clear();
  for (int b = 0; b < n_owned; ++b)
  {
    const Key k = out.owned[b];
    // only a leaf on a non-periodic border has outside neighbours
    const int kc[3] = {k.x, k.y, k.z};
    bool      border = false;
    for (int d = 0; d < f.dim; ++d)
      border = border || (!f.per[d] && (kc[d] == 0 || kc[d] == f.ext(k.L, d) - 1));
    if (!border)
      continue;
    for (int o = 0; o < f.noffs; ++o)
    {
      int c[3] = {k.x + f.offs[o][0], k.y + f.offs[o][1], k.z + f.offs[o][2]};
      int w[3] = {c[0], c[1], c[2]};
      if (f.wrap(k.L, w))
        continue;
      for (int d = 0; d < 3; ++d)
        if (f.per[d])
          w[d] = Forest::periodic(c[d], f.ext(k.L, d));
        else
          w[d] = c[d];
      // outside coordinates can be -1: keep them in a separate map keyed by the signed triple
      const uint64_t ok = pack(k.L, w[0] + 1, w[1] + 1, w[2] + 1);
      if (out_ids.contains(ok))
        continue;
      int src[3];
      for (int d = 0; d < 3; ++d)
        src[d] = std::min(std::max(w[d], 0), f.ext(k.L, d) - 1);
      const int32_t * it = ids.find(pack(k.L, src[0], src[1], src[2]));
      if (!it)
      {
        out.n_owned = -1; // an outside block without a same-level inside block
        return;
      }
      out_ids.put(ok, n_owned + (int32_t)out_keys.size());
      out_keys.push_back(Key{k.L, w[0], w[1], w[2]});
      out.out_src.push_back(*it);
      for (int d = 0; d < 3; ++d)
        out.out_normal.push_back(src[d] > w[d] ? 1 : (src[d] < w[d] ? -1 : 0));
    }
  }
  const int n_blocks = n_owned + (int)out_keys.size();
  out.n_owned = n_owned;
  out.n_blocks = n_blocks;
  out.level.assign(n_blocks, 0);
  out.coord.assign((size_t)n_blocks * 3, 0);
  out.neighbor.assign((size_t)n_blocks * 27, -1);
  out.fine_at.clear();
  out.fine_id.clear();
  for (int b = 0; b < n_blocks; ++b)
  {
    const Key k = b < n_owned ? out.owned[b] : out_keys[b - n_owned];
    out.level[b] = k.L;
    out.coord[3 * b] = k.x;
    out.coord[3 * b + 1] = k.y;
    out.coord[3 * b + 2] = k.z;
  }
  // neighbour tables, the owned blocks in ranges over host threads (lookups only; the children found
  // are gathered per range, in block order)
  constexpr int                     MAXT = 16;
  std::vector<std::vector<int64_t>> fat(MAXT);
  std::vector<std::vector<int32_t>> fid(MAXT);
  std::vector<char>                 bad(MAXT, 0);
  const int nt = for_ranges(n_owned, [&](int t, int lo, int hi) {
    for (int b = lo; b < hi && !bad[t]; ++b)
    {
      const Key k = out.owned[b];
      out.neighbor[(size_t)b * 27 + 13] = b; // the block itself
      for (int o = 0; o < f.noffs; ++o)
      {
        const int s = (f.offs[o][2] + 1) * 9 + (f.offs[o][1] + 1) * 3 + (f.offs[o][0] + 1);
        int       r[3] = {k.x + f.offs[o][0], k.y + f.offs[o][1], k.z + f.offs[o][2]};
        int       c[3] = {r[0], r[1], r[2]};
        if (!f.wrap(k.L, r))
        {
          int w[3];
          for (int d = 0; d < 3; ++d)
            w[d] = f.per[d] ? Forest::periodic(c[d], f.ext(k.L, d)) : c[d];
          out.neighbor[(size_t)b * 27 + s] = *out_ids.find(pack(k.L, w[0] + 1, w[1] + 1, w[2] + 1));
          continue;
        }
        const int32_t * it = ids.find(pack(k.L, r[0], r[1], r[2]));
        if (it)
        {
          out.neighbor[(size_t)b * 27 + s] = *it;
          continue;
        }
        if (k.L >= 1 && (it = ids.find(pack(k.L - 1, r[0] >> 1, r[1] >> 1, r[2] >> 1))))
        {
          out.neighbor[(size_t)b * 27 + s] = *it;
          continue;
        }
        bool      found = false;
        const Key rk{k.L, r[0], r[1], r[2]};
        for (int ch = 0; ch < f.nkids(); ++ch)
          if ((it = ids.find(f.kid(rk, ch))))
          {
            fat[t].push_back(((int64_t)b * 27 + s) * 8 + ch);
            fid[t].push_back(*it);
            found = true;
          }
        if (!found)
        {
          bad[t] = 1; // not 2:1 balanced
          break;
        }
      }
    }
  });
  for (int t = 0; t < nt; ++t)
  {
    if (bad[t])
    {
      out.n_owned = -2;
      return;
    }
    out.fine_at.insert(out.fine_at.end(), fat[t].begin(), fat[t].end());
    out.fine_id.insert(out.fine_id.end(), fid[t].begin(), fid[t].end());
  }
  out.has_fine = !out.fine_at.empty();
}

} // namespace

extern "C" {

gmhd_forest *
gmhd_forest_build(int32_t dim, const int32_t * bricks, const int32_t * periodic, int32_t bx, int32_t by, int32_t bz,
                  int32_t level_min, int32_t level_max, int32_t n_leaves, const int32_t * keys, const int8_t * flags)
{
  if ((dim != 2 && dim != 3) || !bricks || !periodic || n_leaves <= 0 || !keys || level_min < 0 ||
      level_max < level_min || level_max > 18 || bx < 4 || by < 4 || (dim == 3 && bz < 4) || bx % 2 || by % 2 ||
      (dim == 3 && bz % 2))
    return nullptr;
  gmhd_forest * out = new (std::nothrow) gmhd_forest();
  if (!out)
    return nullptr;
  Forest f;
  f.dim = dim;
  for (int d = 0; d < 3; ++d)
  {
    f.bricks[d] = d < dim ? bricks[d] : 1;
    f.per[d] = d < dim ? (periodic[d] != 0) : 1;
    if (f.bricks[d] < 1)
    {
      delete out;
      return nullptr;
    }
  }
  f.base = level_min;
  f.init();
  out->dim = dim;
  out->bx = bx;
  out->by = by;
  out->bz = dim == 3 ? bz : 1;
  std::vector<uint64_t> old(n_leaves);
  KeyTable              old_id(n_leaves);
  for (int n = 0; n < n_leaves; ++n)
  {
    const int32_t * k = keys + 4 * n;
    if (k[0] < 0 || k[0] > 18 || k[1] < 0 || k[2] < 0 || k[3] < 0)
    {
      delete out;
      return nullptr;
    }
    old[n] = pack(k[0], k[1], k[2], dim == 3 ? k[3] : 0);
    old_id.put(old[n], n);
  }
  KeyTable cand(n_leaves);
  if (flags)
  {
    // refine flagged leaves, coarsen whole flagged families; undo a coarsening that balance refines again
    std::vector<uint64_t> refined, coarsen;
    KeyTable              family;
    for (int n = 0; n < n_leaves; ++n)
    {
      const Key k = unpack(old[n]);
      if (flags[n] > 0 && k.L < level_max)
        refined.push_back(old[n]);
      else if (flags[n] < 0 && k.L > level_min)
      {
        const uint64_t  p = pack(k.L - 1, k.x >> 1, k.y >> 1, k.z >> 1);
        const int32_t * c = family.find(p);
        family.put(p, c ? *c + 1 : 1);
      }
    }
    family.for_each([&](uint64_t p, int32_t c) {
      if (c == f.nkids())
        coarsen.push_back(p);
    });
    std::sort(coarsen.begin(), coarsen.end());
    while (true)
    {
      cand = KeyTable(n_leaves + refined.size() * f.nkids());
      for (uint64_t kk : old)
        cand.put(kk);
      for (uint64_t kk : refined)
      {
        cand.erase(kk);
        for (int c = 0; c < f.nkids(); ++c)
          cand.put(f.kid(unpack(kk), c));
      }
      for (uint64_t p : coarsen)
      {
        for (int c = 0; c < f.nkids(); ++c)
          cand.erase(f.kid(unpack(p), c));
        cand.put(p);
      }
      // the input set is balanced (it comes from an earlier build): only new children and the leaves
      // next to new parents can break the balance
      std::vector<uint64_t> seeds;
      for (uint64_t kk : refined)
        for (int c = 0; c < f.nkids(); ++c)
          seeds.push_back(f.kid(unpack(kk), c));
      for (uint64_t p : coarsen)
        f.fine_neighbours_of(cand, p, seeds);
      f.balance(cand, &seeds);
      const size_t before = coarsen.size();
      coarsen.erase(std::remove_if(coarsen.begin(), coarsen.end(), [&](uint64_t p) { return !cand.contains(p); }),
                    coarsen.end());
      if (coarsen.size() == before)
        break;
    }
  }
  else
  {
    for (uint64_t kk : old)
      cand.put(kk);
    f.balance(cand);
  }
  build(f, cand, *out);
  if (out->n_owned < 0)
  {
    delete out;
    return nullptr;
  }
  // remap rows: kind, sources, kept same-level leaves across the faces
  out->remap.assign((size_t)out->n_owned * 15, -1);
  for (int n = 0; n < out->n_owned; ++n)
  {
    int32_t * rm = &out->remap[(size_t)n * 15];
    const Key k = out->owned[n];
    const uint64_t kk = pack(k.L, k.x, k.y, k.z);
    const int32_t * it = old_id.find(kk);
    if (it)
    {
      rm[0] = 0;
      rm[1] = *it;
      continue;
    }
    if (k.L >= 1 && (it = old_id.find(pack(k.L - 1, k.x >> 1, k.y >> 1, k.z >> 1))))
    {
      rm[0] = 1;
      rm[1] = *it;
      rm[2] = (k.x & 1) + 2 * (k.y & 1) + 4 * (k.z & 1);
    }
    else
    {
      rm[0] = 2;
      for (int c = 0; c < f.nkids(); ++c)
      {
        it = old_id.find(f.kid(k, c));
        rm[1 + c] = it ? *it : -1;
      }
    }
    for (int fc = 0; fc < 2 * dim; ++fc)
    {
      int r[3] = {k.x, k.y, k.z};
      r[fc / 2] += fc % 2 == 0 ? -1 : 1;
      if (!f.wrap(k.L, r))
        continue;
      const uint64_t rk = pack(k.L, r[0], r[1], r[2]);
      const int32_t * kept = old_id.find(rk);
      if (kept && cand.contains(rk))
        rm[9 + fc] = *kept;
    }
  }
  return out;
}

int
gmhd_forest_sizes(const gmhd_forest * f, int32_t * n_owned, int32_t * n_blocks, int32_t * has_fine)
{
  if (!f || !n_owned || !n_blocks)
    return GMHD_ERR_ARGUMENT;
  *n_owned = f->n_owned;
  *n_blocks = f->n_blocks;
  if (has_fine)
    *has_fine = f->has_fine ? 1 : 0;
  return GMHD_OK;
}

int
gmhd_forest_tables(const gmhd_forest * f, int32_t * level, int32_t * coord, int32_t * neighbor, int32_t * fine_neighbor,
                   int32_t * outside_src, int32_t * outside_normal, int32_t * remap)
{
  if (!f)
    return GMHD_ERR_ARGUMENT;
  auto put = [](int32_t * dst, const std::vector<int32_t> & src) {
    if (dst && !src.empty())
      std::memcpy(dst, src.data(), src.size() * sizeof(int32_t));
  };
  put(level, f->level);
  put(coord, f->coord);
  put(neighbor, f->neighbor);
  if (fine_neighbor)
  {
    std::memset(fine_neighbor, 0xff, sizeof(int32_t) * (size_t)f->n_blocks * 27 * 8);
    for (size_t i = 0; i < f->fine_at.size(); ++i)
      fine_neighbor[f->fine_at[i]] = f->fine_id[i];
  }
  put(outside_src, f->out_src);
  put(outside_normal, f->out_normal);
  put(remap, f->remap);
  return GMHD_OK;
}

int
gmhd_forest_fine(const gmhd_forest * f, int64_t * n_fine, int64_t * at, int32_t * id)
{
  if (!f || !n_fine)
    return GMHD_ERR_ARGUMENT;
  *n_fine = (int64_t)f->fine_at.size();
  if (at && !f->fine_at.empty())
    std::memcpy(at, f->fine_at.data(), f->fine_at.size() * sizeof(int64_t));
  if (id && !f->fine_id.empty())
    std::memcpy(id, f->fine_id.data(), f->fine_id.size() * sizeof(int32_t));
  return GMHD_OK;
}

void
gmhd_forest_destroy(gmhd_forest * f)
{
  delete f;
}

} // extern "C"
