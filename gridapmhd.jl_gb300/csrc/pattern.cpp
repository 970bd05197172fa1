// CSR sparsity pattern of the Newton Jacobian and the cell -> nonzero map.
//
// Restates the symbolic phase of Gridap's SparseMatrixAssembler for the
// consecutive [u;p;j;φ] layout (GridapMHD src/main.jl:218-224): every block
// touched by the Jacobian integrand (uu, up, uj, pu, jj, jφ, ju, φj;
// src/weakforms.jl:283-312) contributes its full element block; Dirichlet rows
// and columns are dropped; columns are sorted inside each row.
//
// The map stores, for every (cell, local row a, local column b), the offset of
// the column inside row a.  Cells whose offset tables are identical (all
// interior cells of a structured mesh with a structured numbering) share one
// table ("class"), so the map read by the assembly kernel stays in L2.
#include <algorithm>
#include <cstring>
#include <unordered_map>

#include "internal.h"

namespace gbmhd {

static inline int field_of(int a) { return a < OP ? 0 : (a < OJ ? 1 : (a < OPHI ? 2 : 3)); }

bool touched(int a, int b) {
  static const bool T[4][4] = {{true, true, true, false},
                               {true, false, false, false},
                               {true, false, true, true},
                               {false, false, true, false}};
  return T[field_of(a)][field_of(b)];
}

static uint64_t fnv1a(const uint16_t* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char* c = reinterpret_cast<const unsigned char*>(p);
  for (size_t i = 0; i < 2 * n; ++i) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
  return h;
}

std::string build_pattern(int64_t ncells, int64_t ndofs, const int32_t* cell_row, Pattern& P) {
  P.n = ndofs;
  // row -> (cell, local) incidence
  std::vector<int64_t> inc_ptr(ndofs + 1, 0);
  for (int64_t c = 0; c < ncells; ++c)
    for (int a = 0; a < ND; ++a) {
      int32_t r = cell_row[c * ND + a];
      if (r >= 0) {
        if (r >= ndofs) return "cell dof id out of range";
        inc_ptr[r + 1]++;
      }
    }
  for (int64_t r = 0; r < ndofs; ++r) inc_ptr[r + 1] += inc_ptr[r];
  std::vector<int64_t> inc(inc_ptr[ndofs]);
  {
    std::vector<int64_t> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int64_t c = 0; c < ncells; ++c)
      for (int a = 0; a < ND; ++a) {
        int32_t r = cell_row[c * ND + a];
        if (r >= 0) inc[fill[r]++] = c * ND + a;
      }
  }
  for (int64_t r = 0; r < ndofs; ++r)
    if (inc_ptr[r + 1] == inc_ptr[r]) return "a free dof belongs to no cell";
  // the sorted distinct columns of row r: candidates from the row's cells, de-duplicated
  // with a per-thread stamp array (one entry per dof) before the sort, so the sort sees
  // each column once instead of once per cell that shares it
  auto row_columns = [&](int64_t r, std::vector<int32_t>& stamp, std::vector<int32_t>& buf) {
    buf.clear();
    for (int64_t k = inc_ptr[r]; k < inc_ptr[r + 1]; ++k) {
      const int64_t c = inc[k] / ND;
      const int a = (int)(inc[k] % ND);
      for (int b = 0; b < ND; ++b) {
        const int32_t cb = cell_row[c * ND + b];
        if (cb >= 0 && stamp[cb] != (int32_t)r && touched(a, b)) {
          stamp[cb] = (int32_t)r;
          buf.push_back(cb);
        }
      }
    }
    std::sort(buf.begin(), buf.end());
  };
  // row lengths
  std::vector<int64_t> len(ndofs, 0);
#pragma omp parallel
  {
    std::vector<int32_t> buf, stamp(ndofs, -1);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t r = 0; r < ndofs; ++r) {
      row_columns(r, stamp, buf);
      len[r] = (int64_t)buf.size();
    }
  }
  P.rowptr.assign(ndofs + 1, 0);
  for (int64_t r = 0; r < ndofs; ++r) P.rowptr[r + 1] = P.rowptr[r] + len[r];
  P.nnz = P.rowptr[ndofs];
  for (int64_t r = 0; r < ndofs; ++r)
    if (len[r] >= 65535) return "row too long for the 16-bit cell map";
  P.col.resize(P.nnz);
#pragma omp parallel
  {
    std::vector<int32_t> buf, stamp(ndofs, -1);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t r = 0; r < ndofs; ++r) {
      row_columns(r, stamp, buf);
      std::copy(buf.begin(), buf.end(), P.col.begin() + P.rowptr[r]);
    }
  }
  // cell map with class de-duplication
  const size_t TS = (size_t)ND * ND;
  // offsets of the cell's columns inside each of its rows: the cell's (column, slot) pairs
  // are sorted once, then each row is walked once alongside them (a merge instead of a
  // binary search per entry); entries of untouched blocks are 0xFFFF
  auto cell_table = [&](int64_t c, uint16_t* t) {
    std::pair<int32_t, int> cb[ND];
    int m = 0;
    for (int b = 0; b < ND; ++b)
      if (cell_row[c * ND + b] >= 0) cb[m++] = {cell_row[c * ND + b], b};
    std::sort(cb, cb + m);
    for (int a = 0; a < ND; ++a) {
      uint16_t* ta = t + (size_t)a * ND;
      std::fill(ta, ta + ND, (uint16_t)0xFFFF);
      const int32_t ra = cell_row[c * ND + a];
      if (ra < 0) continue;
      const int32_t* beg = P.col.data() + P.rowptr[ra];
      const int32_t* end = P.col.data() + P.rowptr[ra + 1];
      const int32_t* q = beg;
      for (int i = 0; i < m; ++i) {
        while (q < end && *q < cb[i].first) ++q;
        if (touched(a, cb[i].second)) ta[cb[i].second] = (uint16_t)(q - beg);
      }
    }
  };
  std::vector<uint64_t> hash(ncells);
#pragma omp parallel
  {
    std::vector<uint16_t> t(TS);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < ncells; ++c) {
      cell_table(c, t.data());
      hash[c] = fnv1a(t.data(), TS);
    }
  }
  std::unordered_map<uint64_t, int32_t> cls;
  std::vector<int64_t> rep;
  P.cell_class.resize(ncells);
  const int32_t kMaxClass = 1 << 16;
  bool per_cell = false;
  for (int64_t c = 0; c < ncells; ++c) {
    auto it = cls.find(hash[c]);
    if (it == cls.end()) {
      if ((int32_t)rep.size() >= kMaxClass) { per_cell = true; break; }
      int32_t id = (int32_t)rep.size();
      cls.emplace(hash[c], id);
      rep.push_back(c);
      P.cell_class[c] = id;
    } else {
      P.cell_class[c] = it->second;
    }
  }
  if (!per_cell) {
    P.nclass = (int32_t)rep.size();
    P.offtab.resize((size_t)P.nclass * TS);
#pragma omp parallel for schedule(static)
    for (int32_t k = 0; k < P.nclass; ++k) cell_table(rep[k], P.offtab.data() + (size_t)k * TS);
    // verify (hash collisions fall back to one table per cell)
    bool ok = true;
#pragma omp parallel
    {
      std::vector<uint16_t> t(TS);
#pragma omp for schedule(static) reduction(&& : ok)
      for (int64_t c = 0; c < ncells; ++c) {
        cell_table(c, t.data());
        ok = ok && std::memcmp(t.data(), P.offtab.data() + (size_t)P.cell_class[c] * TS, 2 * TS) == 0;
      }
    }
    if (!ok) per_cell = true;
  }
  if (per_cell) {
    P.nclass = (int32_t)ncells;
    P.offtab.resize((size_t)ncells * TS);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < ncells; ++c) {
      P.cell_class[c] = (int32_t)c;
      cell_table(c, P.offtab.data() + (size_t)c * TS);
    }
  }
  return "";
}

}  // namespace gbmhd
