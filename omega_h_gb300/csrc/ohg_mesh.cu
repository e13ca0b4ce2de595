// Adjacency derivation, box construction, Hilbert renumbering, box
// classification and the measurement kernels.
#include <cfloat>

#include "ohg_math.cuh"
#include "ohg_mesh.cuh"
#include "ohg_screen.cuh"
#include "ohg_workload.hpp"

namespace ohg {

// ------------------------------------------------------------ invert_adj
// key = hl * 8 + down code (packed) or hl with the code read from dc
__device__ __forceinline__ void unpack_use(LO key, int k, LO* lh2hl, I8* codes, LO j,
                                           const I8* dc, bool packed) {
  LO hl = packed ? key >> 3 : key;
  int c = packed ? (key & 7) : (dc ? int(dc[hl] & 7) : 0);
  codes[j] = make_code(c & 1, (c >> 1) & 3, hl % k);
  lh2hl[j] = hl / k;
}

// One launch for every row length, with no host read of the longest row:
// each warp takes four consecutive rows.  When all four have at most 8
// entries (a warp vote), 8-lane groups sort them at once; when all have at
// most 16, half warps sort them two at a time; otherwise the whole warp sorts
// them one after the other with 1, 2 or 4 entries per lane (rows beyond 128
// entries by one lane in memory).  Every branch is uniform across
// the warp, so the shuffles always run on full warps.
template <int E>
__device__ __forceinline__ void warp_sort_row(LO b, LO n, int lane, LO* lh2hl, I8* codes, int k,
                                              const I8* dc, bool packed) {
  constexpr int G = 32;
  LO v[E];
#pragma unroll
  for (int r = 0; r < E; ++r) {
    int i = r * G + lane;
    v[r] = (i < n) ? lh2hl[b + i] : 0x7fffffff;
  }
  for (int kk = 2; kk <= G * E; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      if (j >= G) {
        int jr = j / G;
#pragma unroll
        for (int jc = 1; jc < E; jc <<= 1) {
          if (jr != jc) continue;
#pragma unroll
          for (int r = 0; r < E; ++r) {
            const int p = r ^ jc;
            if (p > r && p < E) {
              int i = r * G + lane;
              bool up = (i & kk) == 0;
              LO x = v[r], y = v[p];
              v[r] = up ? min(x, y) : max(x, y);
              v[p] = up ? max(x, y) : min(x, y);
            }
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          LO o = __shfl_xor_sync(0xffffffffu, v[r], j);
          int i = r * G + lane;
          bool up = (i & kk) == 0;
          bool lower = (lane & j) == 0;
          v[r] = (lower == up) ? min(v[r], o) : max(v[r], o);
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < E; ++r) {
    int i = r * G + lane;
    if (i < n) unpack_use(v[r], k, lh2hl, codes, b + i, dc, packed);
  }
}

// a row of at most G entries sorted by a group of G lanes (sl = lane in group)
template <int G>
__device__ __forceinline__ void group_sort_row(LO b, LO n, int sl, LO* lh2hl, I8* codes, int k,
                                               const I8* dc, bool packed) {
  LO v = sl < n ? lh2hl[b + sl] : 0x7fffffff;
#pragma unroll
  for (int kk = 2; kk <= G; kk <<= 1) {
#pragma unroll
    for (int j = kk >> 1; j > 0; j >>= 1) {
      LO o = __shfl_xor_sync(0xffffffffu, v, j, G);
      bool up = (sl & kk) == 0;
      bool lower = (sl & j) == 0;
      v = (lower == up) ? min(v, o) : max(v, o);
    }
  }
  if (sl < n) unpack_use(v, k, lh2hl, codes, b + sl, dc, packed);
}

__global__ void k_row_sort_adaptive(LO nlows, const LO* off, LO* lh2hl, I8* codes, int k,
                                    const I8* dc, bool packed) {
  unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  int lane = int(t & 31u);
  LO row0 = LO(t >> 5) * 4;
  LO l = row0 + (lane >> 3);
  LO b = l < nlows ? off[l] : 0, n = l < nlows ? off[l + 1] - b : 0;
  if (!__any_sync(0xffffffffu, n > 8)) {
    // four rows of at most 8 entries, one per 8-lane group
    group_sort_row<8>(b, n, lane & 7, lh2hl, codes, k, dc, packed);
    return;
  }
  if (!__any_sync(0xffffffffu, n > 16)) {
    // two rows at a time of at most 16 entries, one per half warp
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      LO l2 = row0 + 2 * h + (lane >> 4);
      LO b2 = l2 < nlows ? off[l2] : 0, n2 = l2 < nlows ? off[l2 + 1] - b2 : 0;
      group_sort_row<16>(b2, n2, lane & 15, lh2hl, codes, k, dc, packed);
    }
    return;
  }
  for (int r = 0; r < 4; ++r) {
    LO row = row0 + r;
    if (row >= nlows) break;  // same for every lane
    LO rb = off[row], rn = off[row + 1] - rb;
    if (rn <= 32) {
      warp_sort_row<1>(rb, rn, lane, lh2hl, codes, k, dc, packed);
    } else if (rn <= 64) {
      warp_sort_row<2>(rb, rn, lane, lh2hl, codes, k, dc, packed);
    } else if (rn <= 128) {
      warp_sort_row<4>(rb, rn, lane, lh2hl, codes, k, dc, packed);
    } else if (lane == 0) {
      for (LO j = rb + 1; j < rb + rn; ++j) {
        LO x = lh2hl[j];
        LO i = j - 1;
        while (i >= rb && lh2hl[i] > x) {
          lh2hl[i + 1] = lh2hl[i];
          --i;
        }
        lh2hl[i + 1] = x;
      }
      for (LO j = rb; j < rb + rn; ++j) unpack_use(lh2hl[j], k, lh2hl, codes, j, dc, packed);
    }
    __syncwarp();
  }
}

static void sort_rows_by_high(LO nlows, const Arr<LO>& off, Arr<LO>& lh2hl, Arr<I8>& codes, int k,
                              const I8* dc, bool packed) {
  if (nlows <= 0) return;
  Ctx& c = ctx();
  long long nwarps = (nlows + 3) / 4;
  long long nthreads = nwarps * 32;
  if (nthreads + kBlock > 0xffffffffLL) throw Error(8, "invert_adj: too many rows for one launch");
  unsigned nblocks = unsigned((nthreads + kBlock - 1) / kBlock);
  k_row_sort_adaptive<<<nblocks, kBlock, 0, c.stream>>>(nlows, off.data(), lh2hl.data(),
                                                        codes.data(), k, dc, packed);
  ++c.launches;
#ifdef OHG_CHECKED
  checked_after_launch(__FILE__, __LINE__);
#endif
}

// Upward adjacency from a downward one (src/Omega_h_adj.cpp:231-263).
// Degrees by atomics, offsets by scan, slots by atomics, then each row is
// sorted by the high entity's use index so rows list high entities in
// increasing order, the order the reference obtains with sort_by_high_index.
Adj invert_adj(const Adj& down, int k, LO nlows, bool sorted) {
  LO nhl = down.ab2b.size();
  Arr<LO> deg = fill<LO>(nlows, 0);
  auto hl2l = cview(down.ab2b);
  auto dg = view(deg);
  // each use's rank within its row is the count's atomic return value, kept
  // for the fill (one round of atomics instead of two)
  Arr<LO> rank(nhl);
  auto rk = view(rank);
  pfor(nhl, [=] __device__(LO hl) { rk[hl] = atomicAdd(&dg[hl2l[hl]], 1); });
  Adj up;
  up.a2ab = offset_scan(deg);
  up.has_a2ab = true;
  up.ab2b = Arr<LO>(nhl);
  up.codes = Arr<I8>(nhl);
  up.has_codes = true;
  // each slot holds the use index hl and the use's down code (flip,
  // rotation) packed as hl * 8 + code, read here where the reads of the down
  // arrays are coalesced (beyond 2^28 uses the key is hl alone and the code
  // is read afterwards)
  bool packed = nhl < (1 << 28);
  auto off = cview(up.a2ab);
  auto rc = cview(rank);
  auto lh2hl = view(up.ab2b);
  bool has_dc = down.has_codes;
  auto dc = cview(down.codes);
  if (!sorted) {
    // rows in atomic order: each slot gets its final entry and code here
    auto uc = view(up.codes);
    pfor(nhl, [=] __device__(LO hl) {
      LO l = hl2l[hl];
      int c = has_dc ? int(dc[hl] & 7) : 0;
      LO j = off[l] + rc[hl];
      lh2hl[j] = hl / k;
      uc[j] = make_code(c & 1, (c >> 1) & 3, hl % k);
    });
    return up;
  }
  pfor(nhl, [=] __device__(LO hl) {
    LO l = hl2l[hl];
    LO c = has_dc ? LO(dc[hl] & 7) : 0;
    lh2hl[off[l] + rc[hl]] = packed ? hl * 8 + c : hl;
  });
  // rows sorted by high entity (sort_by_high_index)
  sort_rows_by_high(nlows, up.a2ab, up.ab2b, up.codes, k,
                    packed ? nullptr : (has_dc ? down.codes.data() : nullptr), packed);
  return up;
}

Arr<LO> form_uses(const Arr<LO>& hv2v, LO nh, int hd, int ld) {
  int nvh = hd + 1, nvl = ld + 1, nlh = simplex_degree(hd, ld);
  Arr<LO> uv2v(nh * nlh * nvl);
  auto h = cview(hv2v);
  auto u = view(uv2v);
  pfor(nh * nlh, [=] __device__(LO hu) {
    LO hh = hu / nlh;
    int uu = hu % nlh;
    for (int uv = 0; uv < nvl; ++uv) u[hu * nvl + uv] = h[hh * nvh + down_template(hd, ld, uu, uv)];
  });
  return uv2v;
}

// ------------------------------------------------------------ hashed reflect_down
// The same matches as reflect_down (src/Omega_h_adj.cpp:297-441) without the
// low entities' upward lists: the low entities go into an open-addressing
// table keyed by their sorted vertex tuple (the table holds entity numbers;
// a probe compares the stored entity's vertices), and each use looks up its
// own tuple.  Low entities are unique, so each tuple is stored once.  The
// table has a power-of-two size of at least twice the entity count, so a
// probe sequence meets a free slot within its length; both loops are also
// bounded by the table size.
__device__ __forceinline__ unsigned tuple_hash(const LO* sv, int deg) {
  unsigned h = 0x9e3779b9u;
  for (int j = 0; j < deg; ++j) {
    h ^= unsigned(sv[j]) + 0x7f4a7c15u + (h << 6) + (h >> 2);
    h *= 0x85ebca6bu;
    h ^= h >> 15;
  }
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  return h;
}
__device__ __forceinline__ void sort_tuple(LO* v, int deg) {
  if (v[0] > v[1]) { LO t = v[0]; v[0] = v[1]; v[1] = t; }
  if (deg == 3) {
    if (v[1] > v[2]) { LO t = v[1]; v[1] = v[2]; v[2] = t; }
    if (v[0] > v[1]) { LO t = v[0]; v[0] = v[1]; v[1] = t; }
  }
}

Adj reflect_down_hashed(const Arr<LO>& hv2v, LO nh, const Arr<LO>& lv2v, LO nl, int hd, int ld) {
  Ctx& c = ctx();
  int nvh = hd + 1, nlh = simplex_degree(hd, ld), deg = ld + 1;
  LO na = nh * nlh;
  Adj out;
  out.ab2b = Arr<LO>(na);
  if (ld > 0) {
    out.codes = Arr<I8>(na);
    out.has_codes = true;
  }
  if (na == 0) return out;
  LO tsize = 1;
  while (tsize < 2 * nl || tsize < 64) tsize *= 2;
  Arr<LO> table(tsize);
  OHG_CUDA(cudaMemsetAsync(table.data(), 0xff, size_t(tsize) * sizeof(LO), c.stream));
  unsigned tmask = unsigned(tsize - 1);
  auto tab = view(table);
  auto lv = cview(lv2v);
  int* st = c.d_status;
  pfor(nl, [=] __device__(LO l) {
    LO sv[3];
    for (int j = 0; j < deg; ++j) sv[j] = lv[l * deg + j];
    sort_tuple(sv, deg);
    unsigned slot = tuple_hash(sv, deg) & tmask;
    for (LO probe = 0; probe <= LO(tmask); ++probe) {
      if (atomicCAS(&tab[LO(slot)], -1, l) == -1) return;
      slot = (slot + 1) & tmask;
    }
    raise_status(st, ST_NO_MATCH);  // unreachable with the table at most half full
  });
  auto h = cview(hv2v);
  auto o = view(out.ab2b);
  auto oc = view(out.codes);
  bool with_codes = ld > 0;
  pfor(na, [=] __device__(LO a) {
    LO hh = a / nlh;
    int uu = a % nlh;
    LO av[3], sv[3];
    for (int j = 0; j < deg; ++j) sv[j] = av[j] = h[hh * nvh + down_template(hd, ld, uu, j)];
    sort_tuple(sv, deg);
    unsigned slot = tuple_hash(sv, deg) & tmask;
    for (LO probe = 0; probe <= LO(tmask); ++probe) {
      LO l = tab[LO(slot)];
      if (l < 0) break;
      LO lw[3], ls[3];
      for (int j = 0; j < deg; ++j) ls[j] = lw[j] = lv[l * deg + j];
      sort_tuple(ls, deg);
      bool same = ls[0] == sv[0] && ls[1] == sv[1] && (deg == 2 || ls[2] == sv[2]);
      if (same) {
        o[a] = l;
        if (with_codes) {
          // positions of av[0] and av[1] in the match give the alignment
          int p0 = lw[0] == av[0] ? 0 : lw[1] == av[0] ? 1 : 2;
          I8 code;
          if (deg == 2) {
            code = make_code(false, p0, 0);
          } else {
            int p1 = lw[0] == av[1] ? 0 : lw[1] == av[1] ? 1 : 2;
            code = make_code(p1 != (p0 + 1) % 3, rotation_to_first(3, p0), 0);
          }
          oc[a] = code;
        }
        return;
      }
      slot = (slot + 1) & tmask;
    }
    raise_status(st, ST_NO_MATCH);
    o[a] = 0;
    if (with_codes) oc[a] = 0;
  });
  return out;
}

// reflect_down / find_matches (src/Omega_h_adj.cpp:297-441): one thread per
// use scans the upward list of the use's vertex with the fewest entries.
// With check_unique the whole list is scanned and a second match is an
// error; without it (entities this library built, unique by construction)
// the scan stops at the match.
Adj reflect_down(const Arr<LO>& hv2v, LO nh, const Arr<LO>& lv2v, const Adj& v2l, int hd, int ld,
                 bool check_unique) {
  int nvh = hd + 1, nlh = simplex_degree(hd, ld), deg = ld + 1;
  LO na = nh * nlh;
  Adj out;
  out.ab2b = Arr<LO>(na);
  if (ld > 0) {
    out.codes = Arr<I8>(na);
    out.has_codes = true;
  }
  auto h = cview(hv2v);
  auto lv = cview(lv2v);
  auto va = cview(v2l.a2ab);
  auto vb = cview(v2l.ab2b);
  auto vc = cview(v2l.codes);
  auto o = view(out.ab2b);
  bool with_codes = ld > 0;
  auto oc = view(out.codes);
  int* st = ctx().d_status;
  pfor(na, [=] __device__(LO a) {
    LO hh = a / nlh;
    int uu = a % nlh;
    LO av[3];
    for (int j = 0; j < deg; ++j) av[j] = h[hh * nvh + down_template(hd, ld, uu, j)];
    // The matching low entity contains every vertex of the use, so any of
    // their upward lists finds it; the shortest is scanned.  The alignment
    // code depends only on where av[0] sits in the match.
    int js = 0;
    LO dmin = va[av[0] + 1] - va[av[0]];
    for (int j = 1; j < deg; ++j) {
      LO dj = va[av[j] + 1] - va[av[j]];
      if (dj < dmin) {
        dmin = dj;
        js = j;
      }
    }
    LO fv = av[js];
    int found = 0;
    for (LO x = va[fv]; x < va[fv + 1]; ++x) {
      LO b = vb[x];
      int wj = code_which_down(vc[x]);  // position of av[js] in b
      LO bb = b * deg;
      I8 mc = 0;
      bool match = false;
      if (deg == 2) {
        if (av[1 - js] == lv[bb + (1 - wj)]) {
          mc = make_code(false, js == 0 ? wj : 1 - wj, 0);
          match = true;
        }
      } else {
        // rotate so that av[0] leads: av[0] is at position (wj - js) mod 3
        int wd = (wj - js + 3) % 3;
        if (av[1] == lv[bb + (wd + 1) % 3] && av[2] == lv[bb + (wd + 2) % 3] &&
            av[0] == lv[bb + wd]) {
          mc = make_code(false, rotation_to_first(3, wd), 0);
          match = true;
        } else {
          // flipped: av = (b[w], b[w-1], b[w-2]) with av[0] at position w;
          // av[js] at wj gives w = wj + js
          int wf = (wj + js) % 3;
          if (av[0] == lv[bb + wf] && av[1] == lv[bb + (wf + 2) % 3] &&
              av[2] == lv[bb + (wf + 1) % 3]) {
            mc = make_code(true, rotation_to_first(3, wf), 0);
            match = true;
          }
        }
      }
      if (match) {
        ++found;
        o[a] = b;
        if (with_codes) oc[a] = mc;
        if (!check_unique) break;
      }
    }
    if (found != 1) {
      raise_status(st, ST_NO_MATCH);
      if (!found) {
        o[a] = 0;
        if (with_codes) oc[a] = 0;
      }
    }
  });
  return out;
}

// transit (src/Omega_h_adj.cpp:443-510)
// transit for a fixed (high, low) pair: one thread per high entity reads
// its middle-dimension row once and writes all its low entities, with the
// templates unrolled (the pairs are (2,0), (3,0) and (3,1))
// entities of dimension t on a simplex of dimension f: C(f+1, t+1)
constexpr int simplex_degree_c(int f, int t) {
  return f == 3 ? (t == 0 ? 4 : t == 1 ? 6 : t == 2 ? 4 : 1)
                : f == 2 ? (t == 2 ? 1 : 3) : f == 1 ? (t == 0 ? 2 : 1) : 1;
}
template <int HD, int LD>
static void transit_fixed(const Adj& h2m, const Adj& m2l, LO nh, Adj& out) {
  constexpr int MD = LD + 1;
  constexpr int NMH = simplex_degree_c(HD, MD);
  constexpr int NLM = simplex_degree_c(MD, LD);
  constexpr int NLH = simplex_degree_c(HD, LD);
  static_assert(HD - LD >= 2, "a transit skips at least one dimension");
  auto hm = cview(h2m.ab2b);
  auto hmc = cview(h2m.codes);
  auto ml = cview(m2l.ab2b);
  auto mlc = cview(m2l.codes);
  auto o = view(out.ab2b);
  auto oc = view(out.codes);
  pfor(nh, [=] __device__(LO h) {
    LO mrow[NMH];
    I8 crow[NMH];
#pragma unroll
    for (int i = 0; i < NMH; ++i) {
      mrow[i] = hm[h * NMH + i];
      crow[i] = hmc[h * NMH + i];
    }
#pragma unroll
    for (int hl = 0; hl < NLH; ++hl) {
      UpTemplate ut = up_template0(HD, LD, hl);
      LO m = mrow[ut.up];
      I8 hm2m = invert_alignment(NLM, crow[ut.up]);
      int mli = align_index(NLM, LD, ut.which_down, hm2m);
      o[h * NLH + hl] = ml[m * NLM + mli];
      if (LD == 1) {
        bool f = code_is_flipped(hm2m) ^ (code_rotation(mlc[m * NLM + mli]) == 1) ^ ut.is_flipped;
        oc[h * NLH + hl] = make_code(false, f, 0);
      }
    }
  });
}

Adj transit(const Adj& h2m, const Adj& m2l, int hd, int ld, LO nh) {
  if ((hd == 2 && ld == 0) || (hd == 3 && ld <= 1)) {
    Adj out;
    int nlh = simplex_degree(hd, ld);
    out.ab2b = Arr<LO>(nh * nlh);
    if (ld == 1) {
      out.codes = Arr<I8>(nh * nlh);
      out.has_codes = true;
    }
    if (hd == 2) transit_fixed<2, 0>(h2m, m2l, nh, out);
    else if (ld == 0) transit_fixed<3, 0>(h2m, m2l, nh, out);
    else transit_fixed<3, 1>(h2m, m2l, nh, out);
    return out;
  }
  int md = ld + 1;
  int nmh = simplex_degree(hd, md), nlm = simplex_degree(md, ld), nlh = simplex_degree(hd, ld);
  Adj out;
  out.ab2b = Arr<LO>(nh * nlh);
  bool with_codes = ld == 1;
  if (with_codes) {
    out.codes = Arr<I8>(nh * nlh);
    out.has_codes = true;
  }
  auto hm = cview(h2m.ab2b);
  auto hmc = cview(h2m.codes);
  auto ml = cview(m2l.ab2b);
  auto mlc = cview(m2l.codes);
  auto o = view(out.ab2b);
  auto oc = view(out.codes);
  pfor(nh * nlh, [=] __device__(LO x) {
    LO h = x / nlh;
    int hl = x % nlh;
    UpTemplate ut = up_template0(hd, ld, hl);
    LO m = hm[h * nmh + ut.up];
    I8 hm2m = invert_alignment(nlm, hmc[h * nmh + ut.up]);
    int mli = align_index(nlm, ld, ut.which_down, hm2m);
    o[x] = ml[m * nlm + mli];
    if (with_codes) {
      bool f = code_is_flipped(hm2m) ^ (code_rotation(mlc[m * nlm + mli]) == 1) ^ ut.is_flipped;
      oc[x] = make_code(false, f, 0);
    }
  });
  return out;
}

// ------------------------------------------------------------ stars, dual
static Adj verts_across_edges(const Adj& e2v, const Adj& v2e) {
  Adj g;
  g.a2ab = v2e.a2ab;
  g.has_a2ab = true;
  g.ab2b = Arr<LO>(v2e.ab2b.size());
  auto ev = cview(e2v.ab2b);
  auto ve = cview(v2e.ab2b);
  auto vc = cview(v2e.codes);
  auto o = view(g.ab2b);
  pfor(v2e.ab2b.size(), [=] __device__(LO x) {
    o[x] = ev[ve[x] * 2 + (1 - code_which_down(vc[x]))];
  });
  return g;
}
static Adj edges_across_tris(const Adj& f2e, const Adj& e2f, LO ne) {
  Adj g;
  Arr<LO> deg(ne);
  auto ea = cview(e2f.a2ab);
  auto dg = view(deg);
  pfor(ne, [=] __device__(LO e) { dg[e] = 2 * (ea[e + 1] - ea[e]); });
  g.a2ab = offset_scan(deg);
  g.has_a2ab = true;
  g.ab2b = Arr<LO>(2 * e2f.ab2b.size());  // two edges per (edge, triangle) use
  auto ga = cview(g.a2ab);
  auto ef = cview(e2f.ab2b);
  auto efc = cview(e2f.codes);
  auto fe = cview(f2e.ab2b);
  auto o = view(g.ab2b);
  pfor(ne, [=] __device__(LO e) {
    LO kk = ga[e];
    for (LO x = ea[e]; x < ea[e + 1]; ++x) {
      LO f = ef[x];
      int ffe = code_which_down(efc[x]);
      o[kk++] = fe[f * 3 + (ffe + 1) % 3];
      o[kk++] = fe[f * 3 + (ffe + 2) % 3];
    }
  });
  return g;
}
static Adj edges_across_tets(const Adj& r2e, const Adj& e2r) {
  Adj g;
  g.a2ab = e2r.a2ab;
  g.has_a2ab = true;
  g.ab2b = Arr<LO>(e2r.ab2b.size());
  auto er = cview(e2r.ab2b);
  auto erc = cview(e2r.codes);
  auto re = cview(r2e.ab2b);
  auto o = view(g.ab2b);
  pfor(e2r.ab2b.size(), [=] __device__(LO x) {
    o[x] = re[er[x] * 6 + opposite_template(3, 1, code_which_down(erc[x]))];
  });
  return g;
}
static Adj add_edges(const Adj& g1, const Adj& g2, LO nv) {
  Adj g;
  Arr<LO> deg(nv);
  auto a1 = cview(g1.a2ab);
  auto a2 = cview(g2.a2ab);
  auto dg = view(deg);
  pfor(nv, [=] __device__(LO v) { dg[v] = (a1[v + 1] - a1[v]) + (a2[v + 1] - a2[v]); });
  g.a2ab = offset_scan(deg);
  g.has_a2ab = true;
  g.ab2b = Arr<LO>(g1.ab2b.size() + g2.ab2b.size());
  auto ga = cview(g.a2ab);
  auto b1 = cview(g1.ab2b);
  auto b2 = cview(g2.ab2b);
  auto o = view(g.ab2b);
  pfor(nv, [=] __device__(LO v) {
    LO kk = ga[v];
    for (LO j = a1[v]; j < a1[v + 1]; ++j) o[kk++] = b1[j];
    for (LO j = a2[v]; j < a2[v + 1]; ++j) o[kk++] = b2[j];
  });
  return g;
}
static Adj elements_across_sides(int dim, const Adj& e2s, const Adj& s2e, LO ne) {
  int nse = dim + 1;
  auto es = cview(e2s.ab2b);
  auto sa = cview(s2e.a2ab);
  auto sb = cview(s2e.ab2b);
  Arr<LO> deg(ne);
  auto dg = view(deg);
  pfor(ne, [=] __device__(LO e) {
    int n = 0;
    for (int k = 0; k < nse; ++k) {
      LO s = es[e * nse + k];
      if (sa[s + 1] - sa[s] >= 2) ++n;
    }
    dg[e] = n;
  });
  Adj g;
  g.a2ab = offset_scan(deg);
  g.has_a2ab = true;
  g.ab2b = Arr<LO>(last(g.a2ab));
  auto ga = cview(g.a2ab);
  auto o = view(g.ab2b);
  pfor(ne, [=] __device__(LO e) {
    LO kk = ga[e];
    for (int k = 0; k < nse; ++k) {
      LO s = es[e * nse + k];
      if (sa[s + 1] - sa[s] >= 2) {
        LO x = sa[s];
        if (sb[x] == e) ++x;
        o[kk++] = sb[x];
      }
    }
  });
  return g;
}

void Mesh::set_ents(int d, Adj down) {
  nents[d] = down.ab2b.size() / simplex_degree(d, d - 1);
  adj[{d, d - 1}] = std::move(down);
  adj_any_order.clear();
}

const Adj& Mesh::ask_up_any_order(int from, int to) {
  auto it = adj.find({from, to});
  if (it != adj.end()) return it->second;
  auto jt = adj_any_order.find({from, to});
  if (jt != adj_any_order.end()) return jt->second;
  if (from < 0 || from >= to || to > dim) throw Error(8, "bad upward adjacency dimensions");
  const Adj& down = ask_adj(to, from);
  return adj_any_order[{from, to}] =
             invert_adj(down, simplex_degree(to, from), nents[from], /*sorted=*/false);
}

void Mesh::drop_cache() {
  adj_any_order.clear();
  for (auto it = adj.begin(); it != adj.end();) {
    if (it->first.second == it->first.first - 1)
      ++it;
    else
      it = adj.erase(it);
  }
}

// An upward adjacency built with its rows in atomic order, put into the
// sorted order: each entry goes back to the key the sorted path sorts (the
// use index hl = high * k + side, packed with the code) and the rows go
// through the same row sort, so the result is the sorted inversion's.
static void sort_any_order_rows(Adj& up, int k, LO nlows, const Adj& down) {
  LO nhl = up.ab2b.size();
  bool packed = nhl < (1 << 28);
  auto ab = view(up.ab2b);
  auto uc = cview(up.codes);
  pfor(nhl, [=] __device__(LO j) {
    I8 c = uc[j];
    LO hl = ab[j] * k + code_which_down(c);
    ab[j] = packed ? hl * 8 + LO(c & 7) : hl;
  });
  sort_rows_by_high(nlows, up.a2ab, up.ab2b, up.codes, k,
                    packed ? nullptr : (down.has_codes ? down.codes.data() : nullptr), packed);
}

// Mesh::derive_adj (src/Omega_h_mesh.cpp:307-345)
const Adj& Mesh::ask_adj(int from, int to) {
  auto it = adj.find({from, to});
  if (it != adj.end()) return it->second;
  if (from < 0 || to < 0 || from > dim || to > dim) throw Error(8, "bad adjacency dimensions");
  Adj d;
  auto jt = from < to ? adj_any_order.find({from, to}) : adj_any_order.end();
  if (jt != adj_any_order.end()) {
    // already inverted for a consumer that ignores row order: sort it
    d = std::move(jt->second);
    adj_any_order.erase(jt);
    sort_any_order_rows(d, simplex_degree(to, from), nents[from], ask_adj(to, from));
    return adj[{from, to}] = std::move(d);
  }
  if (from < to) {
    const Adj& down = ask_adj(to, from);
    d = invert_adj(down, simplex_degree(to, from), nents[from]);
  } else if (to < from) {
    const Adj& h2m = ask_adj(from, to + 1);
    const Adj& m2l = ask_adj(to + 1, to);
    d = transit(h2m, m2l, from, to, nents[from]);
  } else if (from == dim) {
    // a side's other element does not depend on the order of its row
    const Adj& e2s = ask_adj(dim, dim - 1);
    const Adj& s2e = ask_up_any_order(dim - 1, dim);
    d = elements_across_sides(dim, e2s, s2e, nents[dim]);
  } else if (from == VERT) {
    const Adj& e2v = ask_adj(EDGE, VERT);
    const Adj& v2e = ask_adj(VERT, EDGE);
    d = verts_across_edges(e2v, v2e);
  } else {
    const Adj& f2e = ask_adj(FACE, EDGE);
    const Adj& e2f = ask_adj(EDGE, FACE);
    d = edges_across_tris(f2e, e2f, nents[EDGE]);
    if (dim == 3) {
      const Adj& r2e = ask_adj(REGION, EDGE);
      const Adj& e2r = ask_adj(EDGE, REGION);
      Adj t = edges_across_tets(r2e, e2r);
      d = add_edges(d, t, nents[EDGE]);
    }
  }
  return adj[{from, to}] = std::move(d);
}

// ------------------------------------------------------------ find_unique
// (src/Omega_h_adj.cpp:68-153): canonical rotation of each use, stable
// lexicographic sort, keep the last use of each run in its own orientation
Arr<LO> find_unique(const Arr<LO>& hv2v, LO nh, int hd, int ld) {
  Arr<LO> uv2v = form_uses(hv2v, nh, hd, ld);
  int deg = ld + 1;
  LO nu = uv2v.size() / deg;
  Arr<LO> canon(uv2v.size());
  auto u = cview(uv2v);
  auto cn = view(canon);
  pfor(nu, [=] __device__(LO x) {
    LO in[3];
    for (int j = 0; j < deg; ++j) in[j] = u[x * deg + j];
    int min_j = 0;
    LO min_v = in[0];
    for (int j = 1; j < deg; ++j)
      if (in[j] < min_v) {
        min_j = j;
        min_v = in[j];
      }
    int rot = rotation_to_first(deg, min_j);
    LO tmp[3];
    for (int j = 0; j < deg; ++j) tmp[rotate_index(deg, j, rot)] = in[j];
    if (deg == 3 && tmp[2] < tmp[1]) {
      LO t = tmp[1];
      tmp[1] = tmp[2];
      tmp[2] = t;
    }
    for (int j = 0; j < deg; ++j) cn[x * deg + j] = tmp[j];
  });
  Arr<LO> s2u = sort_by_keys(canon, deg);
  Arr<I8> jumps(nu);
  auto s = cview(s2u);
  auto jp = view(jumps);
  auto cnr = cview(canon);
  pfor(nu, [=] __device__(LO i) {
    if (i == nu - 1) {
      jp[i] = 1;
      return;
    }
    LO e0 = s[i], e1 = s[i + 1];
    I8 j = 0;
    for (int k = 0; k < deg; ++k)
      if (cnr[e0 * deg + k] != cnr[e1 * deg + k]) j = 1;
    jp[i] = j;
  });
  Arr<LO> e2s = collect_marked(jumps);
  LO ne = e2s.size();
  Arr<LO> out(ne * deg);
  auto es = cview(e2s);
  auto o = view(out);
  pfor(ne, [=] __device__(LO e) {
    LO uu = s[es[e]];
    for (int k = 0; k < deg; ++k) o[e * deg + k] = u[uu * deg + k];
  });
  return out;
}

// ------------------------------------------------------------ box
// tets_from_hexes (Dompierre et al. case analysis, src/Omega_h_simplify.cpp:20-230)
__device__ __forceinline__ void hex_rot_fwd(LO* v, int n) {
  // the reference's in-place rotation: every slot copies its predecessor's
  // already updated value
  LO tmp = v[n - 1];
  for (int i = 0; i < n - 1; ++i) v[i + 1] = v[i];
  v[0] = tmp;
}
__device__ int hex_case(View<const LO> hv, LO base, LO* hh) {
  for (int i = 0; i < 8; ++i) hh[i] = hv[base + i];
  int min_i = 0;
  for (int i = 1; i < 8; ++i)
    if (hh[i] < hh[min_i]) min_i = i;
  int r = (4 - (min_i % 4)) % 4;
  for (int t = 0; t < r; ++t) hex_rot_fwd(hh, 4);
  for (int t = 0; t < r; ++t) hex_rot_fwd(hh + 4, 4);
  if (min_i >= 4) {
    const int fp[4][2] = {{0, 4}, {3, 5}, {1, 7}, {2, 6}};
    for (int i = 0; i < 4; ++i) {
      LO t = hh[fp[i][0]];
      hh[fp[i][0]] = hh[fp[i][1]];
      hh[fp[i][1]] = t;
    }
  }
  const int bf[3][4] = {{6, 5, 1, 2}, {6, 2, 3, 7}, {6, 7, 4, 5}};
  int di[3];
  for (int i = 0; i < 3; ++i) {
    LO a = min(hh[bf[i][0]], hh[bf[i][2]]), b = min(hh[bf[i][1]], hh[bf[i][3]]);
    di[i] = a < b;
  }
  int nd = di[0] + di[1] + di[2];
  int face = -1;
  if (nd == 1)
    for (int i = 0; i < 3; ++i)
      if (di[i]) face = i;
  if (nd == 2)
    for (int i = 0; i < 3; ++i)
      if (!di[i]) face = i;
  if (face >= 0) {
    const int ring[6] = {1, 2, 3, 7, 5, 4};
    LO tmp[6];
    for (int i = 0; i < 6; ++i) tmp[i] = hh[ring[i]];
    int nt = ((3 - face) % 3) * 2;
    for (int t = 0; t < nt; ++t) hex_rot_fwd(tmp, 6);
    for (int i = 0; i < 6; ++i) hh[ring[i]] = tmp[i];
  }
  return nd;
}
__constant__ int c_hex_tmpl[4][6][4] = {
    {{0, 1, 2, 5}, {0, 2, 7, 5}, {0, 2, 3, 7}, {0, 5, 7, 4}, {2, 7, 5, 6}, {0, 0, 0, 0}},
    {{0, 5, 7, 4}, {0, 1, 7, 5}, {1, 6, 7, 5}, {0, 7, 2, 3}, {0, 7, 1, 2}, {1, 7, 6, 2}},
    {{0, 4, 5, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 1, 2, 5}, {0, 3, 6, 2}, {0, 6, 5, 2}},
    {{0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 5, 6, 4}, {1, 5, 6, 0}, {1, 6, 2, 0}}};

static Arr<LO> box_elems(int dim, int n, Arr<double>* coords) {
  if (dim == 3) {
    LO nvx = n + 1, nvxy = nvx * nvx, nv = nvxy * nvx, nxy = n * n, nh = nxy * n;
    double dx = 1.0 / n;
    *coords = Arr<double>(nv * 3);
    auto c = view(*coords);
    pfor(nv, [=] __device__(LO v) {
      LO ij = v % nvxy, k = v / nvxy, i = ij % nvx, j = ij / nvx;
      c[v * 3 + 0] = i * dx;
      c[v * 3 + 1] = j * dx;
      c[v * 3 + 2] = k * dx;
    });
    Arr<LO> hv(nh * 8);
    auto h = view(hv);
    pfor(nh, [=] __device__(LO x) {
      LO ij = x % nxy, k = x / nxy, i = ij % n, j = ij / n;
      LO b = x * 8;
      h[b + 0] = (k + 0) * nvxy + (j + 0) * nvx + (i + 0);
      h[b + 1] = (k + 0) * nvxy + (j + 0) * nvx + (i + 1);
      h[b + 2] = (k + 0) * nvxy + (j + 1) * nvx + (i + 1);
      h[b + 3] = (k + 0) * nvxy + (j + 1) * nvx + (i + 0);
      h[b + 4] = (k + 1) * nvxy + (j + 0) * nvx + (i + 0);
      h[b + 5] = (k + 1) * nvxy + (j + 0) * nvx + (i + 1);
      h[b + 6] = (k + 1) * nvxy + (j + 1) * nvx + (i + 1);
      h[b + 7] = (k + 1) * nvxy + (j + 1) * nvx + (i + 0);
    });
    Arr<LO> cnt(nh);
    auto ct = view(cnt);
    auto hc = cview(hv);
    pfor(nh, [=] __device__(LO x) {
      LO hh[8];
      ct[x] = hex_case(hc, x * 8, hh) == 0 ? 5 : 6;
    });
    Arr<LO> off = offset_scan(cnt);
    Arr<LO> tv(last(off) * 4);
    auto of = cview(off);
    auto t = view(tv);
    pfor(nh, [=] __device__(LO x) {
      LO hh[8];
      int nd = hex_case(hc, x * 8, hh);
      int nt = nd == 0 ? 5 : 6;
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < 4; ++j) t[(of[x] + i) * 4 + j] = hh[c_hex_tmpl[nd][i][j]];
    });
    return tv;
  }
  LO nvx = n + 1, nv = nvx * nvx, nq = n * n;
  double dx = 1.0 / n;
  *coords = Arr<double>(nv * 2);
  auto c = view(*coords);
  pfor(nv, [=] __device__(LO v) {
    c[v * 2 + 0] = (v % nvx) * dx;
    c[v * 2 + 1] = (v / nvx) * dx;
  });
  Arr<LO> tv(nq * 6);
  auto t = view(tv);
  pfor(nq, [=] __device__(LO q) {
    LO i = q % n, j = q / n;
    // the minimum vertex of a box quad is already first: no rotation
    LO qq[4] = {(j + 0) * nvx + (i + 0), (j + 0) * nvx + (i + 1), (j + 1) * nvx + (i + 1),
                (j + 1) * nvx + (i + 0)};
    const int qt[2][3] = {{0, 1, 2}, {2, 3, 0}};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 3; ++b) t[(q * 2 + a) * 3 + b] = qq[qt[a][b]];
  });
  return tv;
}

static void add_ents2verts(Mesh& m, int d, const Arr<LO>& ev2v, LO ne) {
  if (d == 1) {
    Adj a;
    a.ab2b = ev2v;
    m.set_ents(1, std::move(a));
  } else {
    const Arr<LO>& lv2v = m.ask_verts_of(d - 1);
    const Adj& v2l = m.ask_up(0, d - 1);
    m.set_ents(d, reflect_down(ev2v, ne, lv2v, v2l, d, d - 1));
  }
}

Mesh build_box(int dim, int n) {
  Arr<double> coords;
  Arr<LO> ev2v = box_elems(dim, n, &coords);
  Mesh m;
  m.dim = dim;
  m.nents[0] = coords.size() / dim;
  LO nel = ev2v.size() / (dim + 1);
  for (int md = 1; md < dim; ++md) {
    Arr<LO> mv = find_unique(ev2v, nel, dim, md);
    add_ents2verts(m, md, mv, mv.size() / (md + 1));
  }
  add_ents2verts(m, dim, ev2v, nel);
  m.coords = coords;
  reorder_by_hilbert(m);
  classify_box(m, n);
  // named sets of the box's model entities (get_box_class_sets,
  // src/Omega_h_box.cpp:162-185): the faces (3D) or sides (2D) and the body,
  // by model dimension and id
  if (dim == 3) {
    m.class_sets = {{"z-", {{2, 4}}},  {"y-", {{2, 10}}}, {"x-", {{2, 12}}}, {"body", {{3, 13}}},
                    {"x+", {{2, 14}}}, {"y+", {{2, 16}}}, {"z+", {{2, 22}}}};
  } else {
    m.class_sets = {{"y-", {{1, 1}}}, {"x-", {{1, 3}}}, {"body", {{2, 4}}}, {"x+", {{1, 5}}},
                    {"y+", {{1, 7}}}};
  }
  return m;
}

// ------------------------------------------------------------ Hilbert
// Skilling, "Programming the Hilbert curve" (AIP Conf. Proc. 707, 2004):
// axes -> transpose form, then bit-interleave into dim 64-bit keys
__device__ void hilbert_axes_to_transpose(std::uint64_t* X, int b, int n) {
  std::uint64_t M = std::uint64_t(1) << (b - 1), P, Q, t;
  for (Q = M; Q > 1; Q >>= 1) {
    P = Q - 1;
    for (int i = 0; i < n; i++) {
      if (X[i] & Q)
        X[0] ^= P;
      else {
        t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < n; i++) X[i] ^= X[i - 1];
  t = 0;
  for (Q = M; Q > 1; Q >>= 1)
    if (X[n - 1] & Q) t ^= Q - 1;
  for (int i = 0; i < n; i++) X[i] ^= t;
}

// untranspose (src/Omega_h_hilbert.hpp:112-117): the transposed form's bits,
// most significant first and interleaved across the axes, as dim words of
// b bits each
__device__ void hilbert_untranspose(const std::uint64_t* X, std::uint64_t* Y, int b, int n) {
  for (int j = 0; j < n; ++j) Y[j] = 0;
  for (int i = 0; i < b * n; ++i)
    Y[i / b] |= (((X[i % n] >> (b - 1 - (i / n))) & 1) << (b - 1 - (i % b)));
}

void hilbert_transpose_keys(const std::uint64_t* axes_p, LO n, int dim, int bits,
                            std::uint64_t* keys_p) {
  auto ax = cview(axes_p, n * dim);
  auto k = view(keys_p, n * dim);
  int* st = ctx().d_status;
  pfor(n, [=] __device__(LO i) {
    std::uint64_t X[3], Y[3];
    for (int j = 0; j < dim; ++j) {
      X[j] = ax[i * dim + j];
      if (bits < 64 && (X[j] >> bits) != 0) raise_status(st, ST_BOUNDS);
    }
    hilbert_axes_to_transpose(X, bits, dim);
    hilbert_untranspose(X, Y, bits, dim);
    for (int j = 0; j < dim; ++j) k[i * dim + j] = Y[j];
  });
}

Arr<GO> hilbert_keys(const Arr<double>& coords, LO n, int dim) {
  double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
  for (int j = 0; j < dim; ++j) {
    Arr<double> comp(n);
    auto c = cview(coords);
    auto o = view(comp);
    pfor(n, [=] __device__(LO i) { o[i] = c[i * dim + j]; });
    mn[j] = min_f64(comp);
    mx[j] = max_f64(comp);
  }
  // bounding box made equilateral, affine map into the unit box
  // (src/Omega_h_bbox.hpp:65-79)
  double maxl = mx[0] - mn[0];
  for (int j = 1; j < dim; ++j) maxl = max2d(maxl, mx[j] - mn[j]);
  double s[3] = {0, 0, 0}, t[3] = {0, 0, 0};
  for (int j = 0; j < dim; ++j) {
    double hi = mn[j] + maxl;
    s[j] = 1.0 / (hi - mn[j]);
    t[j] = -(s[j] * mn[j]);
  }
  double s0 = s[0], s1 = s[1], s2 = s[2], t0 = t[0], t1 = t[1], t2 = t[2];
  Arr<GO> keys(n * dim);
  auto c = cview(coords);
  auto k = view(keys);
  pfor(n, [=] __device__(LO i) {
    const int nbits = 52;
    double ss[3] = {s0, s1, s2}, tt[3] = {t0, t1, t2};
    std::uint64_t X[3], Y[3];
    for (int j = 0; j < dim; ++j) {
      double u = ss[j] * c[i * dim + j];
      u = u + tt[j];
      double z = min2d(max2d(u, 0.0), 1.0) * 4503599627370496.0;  // 2^52
      X[j] = std::uint64_t(z);
      if (X[j] >= (std::uint64_t(1) << nbits)) X[j] = (std::uint64_t(1) << nbits) - 1;
    }
    hilbert_axes_to_transpose(X, nbits, dim);
    hilbert_untranspose(X, Y, nbits, dim);
    for (int j = 0; j < dim; ++j) k[i * dim + j] = GO(Y[j]);
  });
  return keys;
}
Arr<LO> hilbert_sort(const Arr<double>& coords, LO n, int dim) {
  return sort_by_keys64(hilbert_keys(coords, n, dim), dim);
}

// reorder_by_hilbert + unmap_mesh (src/Omega_h_reorder.cpp:19-64,
// src/Omega_h_unmap_mesh.cpp:108-136): vertices in Hilbert order, every other
// entity ordered by its first vertex's new number, then by old number
void reorder_by_hilbert(Mesh& m) {
  int dim = m.dim;
  LO nv = m.nverts();
  Arr<LO> new2old[4];
  new2old[0] = hilbert_sort(m.coords, nv, dim);
  Arr<LO> old2new_v(nv);
  {
    auto p = cview(new2old[0]);
    auto o = view(old2new_v);
    pfor(nv, [=] __device__(LO i) { o[p[i]] = i; });
  }
  for (int d = 1; d <= dim; ++d) {
    const Arr<LO>& ev2v = m.ask_verts_of(d);
    int deg = d + 1;
    LO ne = m.nents[d];
    // key = new number of the first vertex; stable sort keeps old order
    Arr<LO> key(ne);
    auto ev = cview(ev2v);
    auto o2n = cview(old2new_v);
    auto kk = view(key);
    pfor(ne, [=] __device__(LO e) { kk[e] = o2n[ev[e * deg]]; });
    new2old[d] = sort_by_keys(key, 1);
  }
  Mesh nm;
  nm.dim = dim;
  nm.nents[0] = nv;
  nm.coords = unmap(new2old[0], m.coords, dim);
  Arr<LO> old2new_low = old2new_v;
  for (int d = 1; d <= dim; ++d) {
    const Adj& od = m.ask_down(d, d - 1);
    int deg = simplex_degree(d, d - 1);
    LO ne = m.nents[d];
    Adj nd;
    nd.ab2b = unmap(new2old[d], od.ab2b, deg);
    auto nb = view(nd.ab2b);
    auto o2n = cview(old2new_low);
    pfor(ne * deg, [=] __device__(LO x) { nb[x] = o2n[nb[x]]; });
    if (od.has_codes) {
      nd.codes = unmap(new2old[d], od.codes, deg);
      nd.has_codes = true;
    }
    nm.set_ents(d, std::move(nd));
    Arr<LO> o2n2(ne);
    auto p = cview(new2old[d]);
    auto o = view(o2n2);
    pfor(ne, [=] __device__(LO i) { o[p[i]] = i; });
    old2new_low = o2n2;
  }
  m = std::move(nm);
}

// classify_box (src/Omega_h_box.cpp:105-160) on the unit square/cube
void classify_box(Mesh& m, int n) {
  int dim = m.dim;
  double dist = 1.0 / double(n * 32);
  for (int d = 0; d <= dim; ++d) {
    LO ne = m.nents[d];
    m.class_id[d] = Arr<LO>(ne);
    m.class_dim[d] = Arr<I8>(ne);
    View<const LO> ev = {nullptr, 0};
    if (d) ev = cview(m.ask_verts_of(d));
    auto c = cview(m.coords);
    auto ci = view(m.class_id[d]);
    auto cd = view(m.class_dim[d]);
    int deg = d + 1;
    pfor(ne, [=] __device__(LO e) {
      int id = 0, cdim = 0;
      for (int j = dim - 1; j >= 0; --j) {
        double x;
        if (d == 0) {
          x = c[e * dim + j];
        } else {
          double comp = 0;
          for (int k = 0; k < deg; ++k) comp += c[ev[e * deg + k] * dim + j];
          comp /= deg;
          x = comp;
        }
        id *= 3;
        if (x > (1.0 - dist)) {
          id += 2;
        } else if (x > dist) {
          id += 1;
          ++cdim;
        }
      }
      ci[e] = id;
      cd[e] = I8(cdim);
    });
  }
}

// seeded jitter of interior vertices and the analytic metric field (host
// side: input construction only)
void apply_workload(Mesh& m, int n, std::uint64_t seed, int kind) {
  bool scalar = workload::scalar_kind(kind);
  int base = workload::base_kind(kind);
  if (scalar && base != workload::METRIC_ISO_LINEAR && base != workload::METRIC_ISO_SINE)
    throw Error(1, "apply_workload: a scalar metric needs an isotropic kind (0 or 3)");
  int dim = m.dim, mc = dim == 3 ? 6 : 3;
  std::vector<double> c = to_host(m.coords);
  std::vector<I8> cd = to_host(m.class_dim[0]);
  LO nv = m.nverts();
  for (LO v = 0; v < nv; ++v) {
    if (cd[v] != dim) continue;
    for (int j = 0; j < dim; ++j) c[size_t(v) * dim + j] += workload::jitter(seed, v, j, dim, n);
  }
  workload::MetricParams mp = workload::make_params(base, seed);
  std::vector<double> met(size_t(nv) * mc);
  for (LO v = 0; v < nv; ++v) workload::metric_at(mp, dim, &c[size_t(v) * dim], &met[size_t(v) * mc]);
  if (scalar) {  // the isotropic tensor's eigenvalue, one per vertex
    for (LO v = 0; v < nv; ++v) met[size_t(v)] = met[size_t(v) * mc];
    met.resize(size_t(nv));
  }
  m.metric_comps = scalar ? 1 : 0;
  m.coords = to_device(c);
  m.metric = to_device(met);
  m.has_length = m.has_quality = false;
  m.screen.reset();
}

// ------------------------------------------------------------ measurement
// measure_edges_metric (src/Omega_h_shape.cpp:7-49): one thread per edge
void measure_edges_metric(Mesh& m, const LO* a2e, LO na, double* out) {
  auto ev = cview(m.ask_verts_of(1));
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  bool all = a2e == nullptr;
  auto ae = cview(a2e, na);
  auto o = view(out, na);
  int dim = m.dim, mc = m.mcomp();
  pfor(na, [=] __device__(LO a) {
    LO e = all ? a : ae[a];
    LO v0 = ev[e * 2], v1 = ev[e * 2 + 1];
    if (mc == 1)
      o[a] = dim == 3 ? edge_length_iso3(&c[v0 * 3], &c[v1 * 3], mt[v0], mt[v1])
                      : edge_length_iso2(&c[v0 * 2], &c[v1 * 2], mt[v0], mt[v1]);
    else
      o[a] = dim == 3 ? edge_length3(&c[v0 * 3], &c[v1 * 3], &mt[v0 * mc], &mt[v1 * mc])
                      : edge_length2(&c[v0 * 2], &c[v1 * 2], &mt[v0 * mc], &mt[v1 * mc]);
  });
}

__device__ __forceinline__ double elem_quality_dev(int dim, int mc, View<const double> c,
                                                   View<const double> mt, const LO* v) {
  double pts[12];
  const double* ms[4];
  for (int i = 0; i <= dim; ++i) {
    for (int j = 0; j < dim; ++j) pts[i * dim + j] = c[v[i] * dim + j];
    ms[i] = &mt[v[i] * mc];
  }
  return elem_quality_ms(dim, mc, pts, ms);
}

// measure_qualities (src/Omega_h_quality.cpp:7-53): one thread per element
void measure_qualities(Mesh& m, const LO* a2e, LO na, double* out) {
  int dim = m.dim, mc = m.mcomp();
  auto ev = cview(m.ask_verts_of(dim));
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  bool all = a2e == nullptr;
  auto ae = cview(a2e, na);
  auto o = view(out, na);
  if (dim == 3 && na > 0) {
    // per-vertex det M (maxdet choice) and sqrt(det M), computed once per
    // vertex instead of four and one times per element: the same doubles
    const VertScreen& vs = mesh_screen(m);
    auto sv = screen_view(vs);
    pfor(na, [=] __device__(LO a) {
      LO e = all ? a : ae[a];
      LO v[4] = {ev[e * 4], ev[e * 4 + 1], ev[e * 4 + 2], ev[e * 4 + 3]};
      o[a] = tet_quality_exact(sv, c, mt, v);
    });
    return;
  }
  pfor(na, [=] __device__(LO a) {
    LO e = all ? a : ae[a];
    LO v[4];
    for (int k = 0; k <= dim; ++k) v[k] = ev[e * (dim + 1) + k];
    o[a] = elem_quality_dev(dim, mc, c, mt, v);
  });
}

// measure_qualities of na elements given by their vertex tuples (dim + 1
// each, in the element's own order): a rebuild's products, whose tuples are
// the rows the new mesh's element-to-vertex list would give them
void measure_qualities_tuples(Mesh& m, const LO* tuples, LO na, double* out) {
  int dim = m.dim, mc = m.mcomp();
  auto tv = cview(tuples, na * (dim + 1));
  auto c = cview(m.coords);
  auto mt = cview(m.metric);
  auto o = view(out, na);
  if (dim == 3 && na > 0) {
    const VertScreen& vs = mesh_screen(m);
    auto sv = screen_view(vs);
    pfor(na, [=] __device__(LO a) {
      LO v[4] = {tv[a * 4], tv[a * 4 + 1], tv[a * 4 + 2], tv[a * 4 + 3]};
      o[a] = tet_quality_exact(sv, c, mt, v);
    });
    return;
  }
  pfor(na, [=] __device__(LO a) {
    LO v[4];
    for (int k = 0; k <= dim; ++k) v[k] = tv[a * (dim + 1) + k];
    o[a] = elem_quality_dev(dim, mc, c, mt, v);
  });
}

// get_mident_metrics (src/Omega_h_metric.cpp:56-104) for edges
void mident_metrics(Mesh& m, const LO* edges, LO n, double* out) {
  auto ev = cview(m.ask_verts_of(1));
  auto mt = cview(m.metric);
  bool all = edges == nullptr;
  auto ed = cview(edges, n);
  int mc = m.mcomp();
  auto o = view(out, n * mc);
  int* st = ctx().d_status;
  if (mc == 1) {
    pfor(n, [=] __device__(LO a) {
      LO e = all ? a : ed[a];
      o[a] = average_metric_iso(mt[ev[e * 2]], mt[ev[e * 2 + 1]]);
    });
  } else if (m.dim == 3 && 2LL * n >= (long long)m.nverts()) {
    // many edges: each vertex's log metric once, then one eigendecomposition
    // per edge instead of three (the same doubles: log_metric3 is a function
    // of the vertex's metric alone)
    LO nv = m.nverts();
    Arr<double> logs(LO(9) * nv);
    auto lg = view(logs);
    pfor(nv, [=] __device__(LO v) {
      double L[9];
      if (!log_metric3(&mt[v * 6], L)) raise_status(st, ST_NUMERIC);
      for (int k = 0; k < 9; ++k) lg[v * 9 + k] = L[k];
    });
    auto lc = cview(logs);
    pfor(n, [=] __device__(LO a) {
      LO e = all ? a : ed[a];
      LO v0 = ev[e * 2], v1 = ev[e * 2 + 1];
      double L0[9], L1[9], r[6];
      for (int k = 0; k < 9; ++k) {
        L0[k] = lc[v0 * 9 + k];
        L1[k] = lc[v1 * 9 + k];
      }
      if (!average_log_metrics3(L0, L1, r)) raise_status(st, ST_NUMERIC);
      for (int k = 0; k < 6; ++k) o[a * 6 + k] = r[k];
    });
  } else if (m.dim == 3) {
    pfor(n, [=] __device__(LO a) {
      LO e = all ? a : ed[a];
      double r[6];
      if (!average_metric3(&mt[ev[e * 2] * 6], &mt[ev[e * 2 + 1] * 6], r)) raise_status(st, ST_NUMERIC);
      for (int k = 0; k < 6; ++k) o[a * 6 + k] = r[k];
    });
  } else {
    pfor(n, [=] __device__(LO a) {
      LO e = all ? a : ed[a];
      double r[3];
      if (!average_metric2(&mt[ev[e * 2] * 3], &mt[ev[e * 2 + 1] * 3], r)) raise_status(st, ST_NUMERIC);
      for (int k = 0; k < 3; ++k) o[a * 3 + k] = r[k];
    });
  }
}

const Arr<double>& Mesh::ask_lengths() {
  if (!has_length) {
    length = Arr<double>(nedges());
    measure_edges_metric(*this, nullptr, nedges(), length.data());
    has_length = true;
  }
  return length;
}
const Arr<double>& Mesh::ask_qualities() {
  if (!has_quality) {
    quality = Arr<double>(nelems());
    measure_qualities(*this, nullptr, nelems(), quality.data());
    has_quality = true;
  }
  return quality;
}

}  // namespace ohg
