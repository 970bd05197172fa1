// CPU test harness: runs the library's build_pattern + mf_analyse (host code) and dumps
// the symbolic structure for the numpy emulation in test_mf_host.py.
#include <cstdio>
#include <string>
#include "mf.h"
using namespace gbmhd;
template <typename V> static void dump(const std::string& dir, const char* name, const std::vector<V>& v) {
  FILE* f = fopen((dir + "/" + name).c_str(), "wb"); fwrite(v.data(), sizeof(V), v.size(), f); fclose(f);
}
extern "C" int mf_harness(int64_t ncells, const double* coords, const int32_t* cell_row, int64_t ndofs, int mono,
                     const char* dir) {
  Pattern P;
  std::string e = build_pattern(ncells, ndofs, cell_row, P);
  if (!e.empty()) { printf("pattern: %s\n", e.c_str()); return 1; }
  MFSymbolic S;
  e = mf_analyse(ncells, coords, cell_row, ndofs, P.rowptr.data(), P.col.data(), mono != 0, S);
  if (!e.empty()) { printf("analyse: %s\n", e.c_str()); return 2; }
  std::string d(dir);
  dump(d, "rowptr", P.rowptr); dump(d, "col", P.col);
  std::vector<int64_t> lev;
  for (auto& L : S.levels) { int64_t a[9] = {L.E, L.B, L.n, L.first, L.count, L.off, L.ah_begin, L.ah_end, L.ch_begin}; lev.insert(lev.end(), a, a + 9); lev.push_back(L.ch_end); }
  dump(d, "levels", lev);
  dump(d, "f_ne", S.f_ne); dump(d, "f_nb", S.f_nb); dump(d, "f_level", S.f_level); dump(d, "f_parent", S.f_parent);
  dump(d, "f_off", S.f_off); dump(d, "elim_ptr", S.elim_ptr); dump(d, "bnd_ptr", S.bnd_ptr); dump(d, "elim", S.elim);
  dump(d, "bnd", S.bnd); dump(d, "ah_src", S.ah_src); dump(d, "ah_dst", S.ah_dst); dump(d, "child_list", S.child_list);
  dump(d, "ea_ptr", S.ea_ptr); dump(d, "ea_pos", S.ea_pos); dump(d, "reg_dst", S.reg_dst); dump(d, "reg_dof", S.reg_dof);
  std::vector<int64_t> sz = {S.storage, (int64_t)S.levels.size(), S.nuj};
  dump(d, "sizes", sz);

  return 0;
}
