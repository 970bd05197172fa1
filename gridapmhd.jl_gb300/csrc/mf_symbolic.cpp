// Symbolic analysis of the (u,j)-block multifrontal factorization (see mf.h).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <numeric>

#include "mf.h"

namespace gbmhd {

namespace {

struct TreeNode {
  int32_t parent = -1;
  int32_t child[2] = {-1, -1};
  int64_t cbeg = 0, cend = 0;   // range in the permuted cell array
  std::vector<int32_t> elim;
  int32_t height = 0;
};

inline bool is_uj_slot(int a) { return a < OP || (a >= OJ && a < OPHI); }
inline int field_of_slot(int a) { return a < OP ? 0 : (a < OJ ? 1 : (a < OPHI ? 2 : 3)); }

}  // namespace

std::string mf_analyse(int64_t ncells, const double* cell_coords, const int32_t* cell_row, int64_t ndofs,
                       const int64_t* rowptr, const int32_t* col, bool monolithic, MFSymbolic& S,
                       int leaf_cells, const char* order) {
  S = MFSymbolic();
  S.monolithic = monolithic;
  auto in_slot = [&](int a) { return monolithic || is_uj_slot(a); };
  std::vector<uint8_t> is_uj(ndofs, 0), kind(ndofs, 0);
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < ND; ++a) {
      const int32_t d = cell_row[c * ND + a];
      if (d < 0) continue;
      kind[d] = (uint8_t)field_of_slot(a);
      if (in_slot(a)) is_uj[d] = 1;
    }
  for (int64_t d = 0; d < ndofs; ++d) S.nuj += is_uj[d];
  // Field order of elimination inside each front (u=0, p=1, j=2, φ=3 ranks).
  int field_rank[4] = {1, 3, 0, 2};  // j, u, φ, p
  if (const char* o = std::getenv("GBMHD_ELIM_ORDER")) order = o;  // diagnostic override
  if (order) {
    // e.g. "jufp": letters in elimination order
    for (int i = 0; order[i] && i < 4; ++i) {
      const int f = order[i] == 'u' ? 0 : order[i] == 'p' ? 1 : order[i] == 'j' ? 2 : 3;
      field_rank[f] = i;
    }
  }
  // cell centres
  std::vector<double> ctr(3 * ncells);
  for (int64_t c = 0; c < ncells; ++c)
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int v = 0; v < 8; ++v) s += cell_coords[24 * c + 3 * v + i];
      ctr[3 * c + i] = s / 8.0;
    }
  std::vector<int32_t> perm(ncells);
  std::iota(perm.begin(), perm.end(), 0);
  std::vector<TreeNode> T;
  T.reserve(4 * ncells / std::max(1, leaf_cells) + 16);
  std::vector<int32_t> assigned(ndofs, -1);
  std::vector<int64_t> stamp(ndofs, -1);
  // breadth-first construction (top-down assignment of separator dofs)
  T.emplace_back();
  T[0].cbeg = 0;
  T[0].cend = ncells;
  for (size_t ni = 0; ni < T.size(); ++ni) {
    const int64_t b = T[ni].cbeg, e = T[ni].cend, n = e - b;
    bool split = false;
    int64_t mid = 0;
    if (n > leaf_cells) {
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int64_t k = b; k < e; ++k)
        for (int i = 0; i < 3; ++i) {
          lo[i] = std::min(lo[i], ctr[3 * perm[k] + i]);
          hi[i] = std::max(hi[i], ctr[3 * perm[k] + i]);
        }
      // split the axis with the most cell layers (distinct centre coordinates), so that a
      // stretched or periodic short direction is not cut before the long ones
      int layers[3] = {0, 0, 0};
      {
        std::vector<double> cs(n);
        for (int i = 0; i < 3; ++i) {
          for (int64_t k = b; k < e; ++k) cs[k - b] = ctr[3 * perm[k] + i];
          std::sort(cs.begin(), cs.end());
          const double tol = 1e-9 * std::max(hi[i] - lo[i], 1e-300);
          int cnt = n > 0 ? 1 : 0;
          for (int64_t k = 1; k < n; ++k)
            if (cs[k] - cs[k - 1] > tol) ++cnt;
          layers[i] = cnt;
        }
      }
      int axes[3] = {0, 1, 2};
      std::sort(axes, axes + 3, [&](int x, int y) {
        return layers[x] != layers[y] ? layers[x] > layers[y] : hi[x] - lo[x] > hi[y] - lo[y];
      });
      for (int ai = 0; ai < 3 && !split; ++ai) {
        const int ax = axes[ai];
        if (hi[ax] - lo[ax] <= 0.0) continue;
        std::stable_sort(perm.begin() + b, perm.begin() + e,
                         [&](int32_t x, int32_t y) { return ctr[3 * x + ax] < ctr[3 * y + ax]; });
        // split at the coordinate change closest to the middle
        const double tol = 1e-9 * (hi[ax] - lo[ax]);
        int64_t best = -1, bestd = n + 1;
        for (int64_t k = b + 1; k < e; ++k)
          if (ctr[3 * perm[k] + ax] - ctr[3 * perm[k - 1] + ax] > tol) {
            int64_t d = std::llabs((k - b) - n / 2);
            if (d < bestd) { bestd = d; best = k; }
          }
        if (best > b && best < e) { split = true; mid = best; }
      }
    }
    if (!split) {
      // leaf: every unassigned (u,j) dof of its cells
      for (int64_t k = b; k < e; ++k) {
        const int64_t c = perm[k];
        for (int a = 0; a < ND; ++a) {
          if (!in_slot(a)) continue;
          const int32_t d = cell_row[c * ND + a];
          if (d >= 0 && assigned[d] < 0) {
            assigned[d] = (int32_t)ni;
            T[ni].elim.push_back(d);
          }
        }
      }
      continue;
    }
    // separator: unassigned dofs touched by both halves
    const int64_t tagL = 2 * (int64_t)ni;
    for (int64_t k = b; k < mid; ++k) {
      const int64_t c = perm[k];
      for (int a = 0; a < ND; ++a)
        if (in_slot(a) && cell_row[c * ND + a] >= 0) stamp[cell_row[c * ND + a]] = tagL;
    }
    for (int64_t k = mid; k < e; ++k) {
      const int64_t c = perm[k];
      for (int a = 0; a < ND; ++a) {
        if (!in_slot(a)) continue;
        const int32_t d = cell_row[c * ND + a];
        if (d >= 0 && stamp[d] == tagL && assigned[d] < 0) {
          assigned[d] = (int32_t)ni;
          T[ni].elim.push_back(d);
        }
      }
    }
    for (int s = 0; s < 2; ++s) {
      TreeNode ch;
      ch.parent = (int32_t)ni;
      ch.cbeg = s == 0 ? b : mid;
      ch.cend = s == 0 ? mid : e;
      T[ni].child[s] = (int32_t)T.size();
      T.push_back(ch);
    }
  }
  for (int64_t d = 0; d < ndofs; ++d)
    if (is_uj[d] && assigned[d] < 0) return "multifrontal analysis left a (u,j) dof unassigned";
  const int64_t nn = (int64_t)T.size();
  if (monolithic) {
    // A subdomain whose boundary velocities and fluxes are not yet eliminated has a
    // constant-pressure (and, with insulating walls, constant-potential) mode: its p and φ
    // Schur pivots are singular.  Each node therefore hands one p dof and one φ dof (the
    // representatives of those modes) up to its parent; only the root keeps the global ones.
    std::vector<int32_t> up_p(nn, -1), up_f(nn, -1);
    for (int64_t v = nn - 1; v >= 0; --v) {
      TreeNode& t = T[v];
      for (int s = 0; s < 2; ++s) {
        const int32_t c = t.child[s];
        if (c < 0) continue;
        for (int32_t d : {up_p[c], up_f[c]})
          if (d >= 0) { t.elim.push_back(d); assigned[d] = (int32_t)v; }
      }
      if (v == 0) break;
      int32_t rp = -1, rf = -1;
      for (int32_t d : t.elim) {
        if (kind[d] == 1 && d > rp) rp = d;
        if (kind[d] == 3 && d > rf) rf = d;
      }
      auto drop = [&](int32_t d) {
        if (d < 0) return;
        t.elim.erase(std::find(t.elim.begin(), t.elim.end(), d));
        assigned[d] = -2;  // re-assigned by the parent
      };
      drop(rp);
      drop(rf);
      up_p[v] = rp;
      up_f[v] = rf;
    }
  }
  // pre-order intervals (children have larger ids than parents: ids are BFS order)
  std::vector<int64_t> pre(nn), last(nn);
  {
    int64_t cnt = 0;
    std::vector<std::pair<int32_t, int>> st;
    st.push_back({0, 0});
    while (!st.empty()) {
      auto& [v, s] = st.back();
      if (s == 0) pre[v] = cnt++;
      if (s < 2 && T[v].child[s] >= 0) {
        int32_t ch = T[v].child[s];
        ++s;
        st.push_back({ch, 0});
      } else if (s < 2) {
        ++s;
      } else {
        last[v] = cnt - 1;
        st.pop_back();
      }
    }
  }
  for (int64_t v = nn - 1; v >= 0; --v)
    for (int s = 0; s < 2; ++s)
      if (T[v].child[s] >= 0) T[v].height = std::max(T[v].height, T[T[v].child[s]].height + 1);
  // boundary sets
  std::vector<std::vector<int32_t>> bnd(nn);
  std::fill(stamp.begin(), stamp.end(), -1);
  for (int64_t v = 0; v < nn; ++v) {
    for (int64_t k = T[v].cbeg; k < T[v].cend; ++k) {
      const int64_t c = perm[k];
      for (int a = 0; a < ND; ++a) {
        if (!in_slot(a)) continue;
        const int32_t d = cell_row[c * ND + a];
        if (d < 0 || stamp[d] == v) continue;
        stamp[d] = v;
        const int64_t p = pre[assigned[d]];
        if (p < pre[v] || p > last[v]) bnd[v].push_back(d);
      }
    }
    std::sort(bnd[v].begin(), bnd[v].end());
    // elimination order inside a front: field rank, then dof id
    std::sort(T[v].elim.begin(), T[v].elim.end(), [&](int32_t x, int32_t y) {
      const int rx = field_rank[kind[x]], ry = field_rank[kind[y]];
      return rx != ry ? rx < ry : x < y;
    });
  }
  // Levels: the fronts of one tree height, in groups of similar size.  A group's fronts share
  // padded sizes E, B and n (the batched kernels need them uniform), so one height whose fronts
  // differ widely in size (irregular 3-D meshes) is split: fronts sorted by size, a group grows
  // while its padded storage stays within 25 % of the fronts' own (at most 8 groups per height).
  // Groups of one height are independent (a front's boundary dofs are eliminated by its
  // ancestors, which are higher), so their order does not matter.
  const int32_t nheight = T[0].height + 1;
  std::vector<std::vector<int32_t>> byh(nheight);
  for (int64_t v = 0; v < nn; ++v) byh[T[v].height].push_back((int32_t)v);
  auto pad8 = [](int64_t x) { return (x + 7) / 8 * 8; };
  std::vector<std::vector<int32_t>> groups;
  for (int32_t h = 0; h < nheight; ++h) {
    std::vector<int32_t>& vs = byh[h];
    std::stable_sort(vs.begin(), vs.end(), [&](int32_t x, int32_t y) {
      return T[x].elim.size() + bnd[x].size() > T[y].elim.size() + bnd[y].size();
    });
    const int64_t total = (int64_t)vs.size();
    std::vector<int32_t> cur;
    int64_t E = 0, B = 0;
    double own = 0.0;
    int made = 0;
    for (int32_t v : vs) {
      const int64_t e = (int64_t)T[v].elim.size(), b = (int64_t)bnd[v].size();
      const int64_t E2 = std::max(E, e), B2 = std::max(B, b);
      const double own2 = own + (double)(e + b) * (double)(e + b);
      const double padded2 = (double)(cur.size() + 1) * (double)(pad8(std::max<int64_t>(E2, 1)) + pad8(B2)) *
                             (double)(pad8(std::max<int64_t>(E2, 1)) + pad8(B2));
      if (!cur.empty() && made < 7 && padded2 > 1.25 * own2 && (int64_t)cur.size() * 16 >= total / 8) {
        groups.push_back(cur);
        ++made;
        cur.clear();
        E = B = 0;
        own = 0.0;
      }
      cur.push_back(v);
      E = std::max(E, e);
      B = std::max(B, b);
      own += (double)(e + b) * (double)(e + b);
    }
    if (!cur.empty()) groups.push_back(cur);
  }
  const int32_t nlev = (int32_t)groups.size();
  std::vector<int32_t> fid(nn), level_of(nn);
  S.levels.resize(nlev);
  int64_t nf = 0, off = 0;
  for (int32_t l = 0; l < nlev; ++l) {
    MFLevel& L = S.levels[l];
    L.first = nf;
    L.count = (int64_t)groups[l].size();
    for (int32_t v : groups[l]) {
      L.E = std::max<int32_t>(L.E, (int32_t)T[v].elim.size());
      L.B = std::max<int32_t>(L.B, (int32_t)bnd[v].size());
      fid[v] = (int32_t)nf++;
      level_of[v] = l;
    }
    // padded to multiples of 8: every front column starts 32-byte aligned, and the sweeps'
    // 16-byte vector loads and TMA boxes stay aligned
    L.E = (std::max(L.E, 1) + 7) / 8 * 8;
    L.B = (L.B + 7) / 8 * 8;
    L.n = L.E + L.B;
    L.off = off;
    off += L.count * (int64_t)L.n * L.n;
    S.flops += (double)L.count * 2.0 * L.n * (double)L.n * L.E;
  }
  S.storage = off;
  S.f_ne.resize(nf); S.f_nb.resize(nf); S.f_level.resize(nf); S.f_parent.assign(nf, -1); S.f_off.resize(nf);
  S.elim_ptr.assign(nf + 1, 0); S.bnd_ptr.assign(nf + 1, 0);
  for (int64_t v = 0; v < nn; ++v) {
    const int32_t f = fid[v];
    const int l = level_of[v];
    S.f_ne[f] = (int32_t)T[v].elim.size();
    S.f_nb[f] = (int32_t)bnd[v].size();
    S.f_level[f] = l;
    S.f_parent[f] = T[v].parent >= 0 ? fid[T[v].parent] : -1;
    S.f_off[f] = S.levels[l].off + (int64_t)(f - S.levels[l].first) * S.levels[l].n * S.levels[l].n;
  }
  std::vector<int32_t> node_of(nf);
  for (int64_t v = 0; v < nn; ++v) node_of[fid[v]] = (int32_t)v;
  for (int64_t f = 0; f < nf; ++f) {
    S.elim_ptr[f + 1] = S.elim_ptr[f] + S.f_ne[f];
    S.bnd_ptr[f + 1] = S.bnd_ptr[f] + S.f_nb[f];
  }
  S.elim.resize(S.elim_ptr[nf]);
  S.bnd.resize(S.bnd_ptr[nf]);
  for (int64_t f = 0; f < nf; ++f) {
    const TreeNode& t = T[node_of[f]];
    std::copy(t.elim.begin(), t.elim.end(), S.elim.begin() + S.elim_ptr[f]);
    std::copy(bnd[node_of[f]].begin(), bnd[node_of[f]].end(), S.bnd.begin() + S.bnd_ptr[f]);
  }
  // arrowheads: the entries of each front's eliminated rows and of its boundary rows in the
  // eliminated columns, front by front (fronts are numbered level by level, so each level's
  // arrowheads are one contiguous range).  Two parallel passes over the fronts: count, then
  // fill at the prefix-summed offsets; the result does not depend on the thread count.
  auto front_arrowheads = [&](int64_t f, std::vector<int32_t>& pos, int32_t* src, int64_t* dst) -> int64_t {
    const MFLevel& L = S.levels[S.f_level[f]];
    const int32_t* el = S.elim.data() + S.elim_ptr[f];
    const int32_t* bd = S.bnd.data() + S.bnd_ptr[f];
    const int ne = S.f_ne[f], nb = S.f_nb[f];
    for (int i = 0; i < ne; ++i) pos[el[i]] = i;
    for (int i = 0; i < nb; ++i) pos[bd[i]] = L.E + i;
    const int64_t base = S.f_off[f];
    int64_t m = 0;
    for (int i = 0; i < ne; ++i) {
      const int32_t e = el[i];
      for (int64_t t = rowptr[e]; t < rowptr[e + 1]; ++t) {
        const int32_t k = col[t];
        if (!is_uj[k] || pos[k] < 0) continue;
        if (src) {
          src[m] = (int32_t)t;
          dst[m] = base + i + (int64_t)pos[k] * L.n;
        }
        ++m;
      }
    }
    for (int i = 0; i < nb; ++i) {
      const int32_t k = bd[i];
      for (int64_t t = rowptr[k]; t < rowptr[k + 1]; ++t) {
        const int32_t c = col[t];
        if (!is_uj[c] || pos[c] < 0 || pos[c] >= L.E) continue;
        if (src) {
          src[m] = (int32_t)t;
          dst[m] = base + (L.E + i) + (int64_t)pos[c] * L.n;
        }
        ++m;
      }
    }
    for (int i = 0; i < ne; ++i) pos[el[i]] = -1;
    for (int i = 0; i < nb; ++i) pos[bd[i]] = -1;
    return m;
  };
  std::vector<int64_t> ah_off(nf + 1, 0);
#pragma omp parallel
  {
    std::vector<int32_t> pos(ndofs, -1);
#pragma omp for schedule(dynamic, 4)
    for (int64_t f = 0; f < nf; ++f) ah_off[f + 1] = front_arrowheads(f, pos, nullptr, nullptr);
  }
  for (int64_t f = 0; f < nf; ++f) ah_off[f + 1] += ah_off[f];
  S.ah_src.resize(ah_off[nf]);
  S.ah_dst.resize(ah_off[nf]);
#pragma omp parallel
  {
    std::vector<int32_t> pos(ndofs, -1);
#pragma omp for schedule(dynamic, 4)
    for (int64_t f = 0; f < nf; ++f)
      front_arrowheads(f, pos, S.ah_src.data() + ah_off[f], S.ah_dst.data() + ah_off[f]);
  }
  for (int32_t l = 0; l < nlev; ++l) {
    S.levels[l].ah_begin = ah_off[S.levels[l].first];
    S.levels[l].ah_end = ah_off[S.levels[l].first + S.levels[l].count];
  }
  // extend-add maps
  S.ea_ptr.assign(nf + 1, 0);
  for (int64_t f = 0; f < nf; ++f) S.ea_ptr[f + 1] = S.ea_ptr[f] + (S.f_parent[f] >= 0 ? S.f_nb[f] : 0);
  S.ea_pos.resize(S.ea_ptr[nf]);
  {
    std::vector<int32_t> pos(ndofs, -1);
    for (int64_t p = 0; p < nf; ++p) {
      const MFLevel& L = S.levels[S.f_level[p]];
      const int32_t* el = S.elim.data() + S.elim_ptr[p];
      const int32_t* bd = S.bnd.data() + S.bnd_ptr[p];
      for (int i = 0; i < S.f_ne[p]; ++i) pos[el[i]] = i;
      for (int i = 0; i < S.f_nb[p]; ++i) pos[bd[i]] = L.E + i;
      const TreeNode& t = T[node_of[p]];
      for (int s = 0; s < 2; ++s) {
        if (t.child[s] < 0) continue;
        const int32_t c = fid[t.child[s]];
        const int32_t* cb = S.bnd.data() + S.bnd_ptr[c];
        for (int i = 0; i < S.f_nb[c]; ++i) {
          if (pos[cb[i]] < 0) return "multifrontal analysis: child boundary not in parent front";
          S.ea_pos[S.ea_ptr[c] + i] = pos[cb[i]];
        }
      }
      for (int i = 0; i < S.f_ne[p]; ++i) pos[el[i]] = -1;
      for (int i = 0; i < S.f_nb[p]; ++i) pos[bd[i]] = -1;
    }
  }
  // children grouped by the level of their parent
  for (int32_t l = 0; l < nlev; ++l) {
    S.levels[l].ch_begin = (int64_t)S.child_list.size();
    for (int64_t f = S.levels[l].first; f < S.levels[l].first + S.levels[l].count; ++f) {
      const TreeNode& t = T[node_of[f]];
      for (int s = 0; s < 2; ++s)
        if (t.child[s] >= 0) S.child_list.push_back(fid[t.child[s]]);
    }
    S.levels[l].ch_end = (int64_t)S.child_list.size();
  }
  if (S.f_nb[S.levels.back().first] != 0) return "multifrontal analysis: root front has a boundary";
  if (monolithic) {
    for (int64_t f = S.levels.back().first; f < S.levels.back().first + S.levels.back().count; ++f) {
      const MFLevel& L = S.levels[S.f_level[f]];
      for (int i = 0; i < S.f_ne[f]; ++i) {
        const int32_t d = S.elim[S.elim_ptr[f] + i];
        if (kind[d] == 1 || kind[d] == 3) {
          S.reg_dst.push_back(S.f_off[f] + i + (int64_t)i * L.n);
          S.reg_dof.push_back(d);
        }
      }
    }
  }
  return "";
}

}  // namespace gbmhd
