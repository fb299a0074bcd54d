// CPU ORACLE — test infrastructure only, never part of the shipped product.
//
// A restatement, in plain C++ with OpenMP, of the reference's CPU algorithm
// for the se_e2_a descriptor path of DeePMD-kit.  Only tests/, the smoke
// check in __graft_entry__.py and bench.py's CPU-baseline leg may load the
// shared library built from this file (liboracle.so).  Each function names
// the reference file:line whose behaviour it follows (paths are relative to
// the reference project root).
//
// Parity pin: this restatement is checked against (1) the golden vectors held
// by the reference's own tests (source/lib/tests/*.cc,
// source/tests/pt/test_tabulate_fusion_se_a.py), extracted into
// tests/golden/*.json, and (2) fixtures produced by the reference's own CPU
// library compiled from its sources (oracle/Makefile -> oracle/_ref/).
//
// Build with -ffp-contract=off: the reference's float32 neighbour sort key
// (r^2 = dx*dx + dy*dy + dz*dz) must not be contracted into FMAs, otherwise
// x86 and aarch64 builds order ties differently.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- region --
// source/lib/src/region.cc:38-80 (compute_volume, compute_rec_boxt) and
// source/lib/src/region.cc:82-113 (tensor_dot_vec / tensor_t_dot_vec).
template <typename T>
T det3_abs(const T* b) {
  T v = b[0] * (b[4] * b[8] - b[7] * b[5]) - b[1] * (b[3] * b[8] - b[6] * b[5]) +
        b[2] * (b[3] * b[7] - b[6] * b[4]);
  return std::abs(v);
}

template <typename T>
void rec_box(T* r, const T* b) {
  T vi = static_cast<T>(1.) / det3_abs(b);
  r[0] = (b[4] * b[8] - b[7] * b[5]) * vi;
  r[4] = (b[0] * b[8] - b[6] * b[2]) * vi;
  r[8] = (b[0] * b[4] - b[3] * b[1]) * vi;
  r[1] = (-b[3] * b[8] + b[6] * b[5]) * vi;
  r[2] = (b[3] * b[7] - b[6] * b[4]) * vi;
  r[3] = (-b[1] * b[8] + b[7] * b[2]) * vi;
  r[5] = (-b[0] * b[7] + b[6] * b[1]) * vi;
  r[6] = (b[1] * b[5] - b[4] * b[2]) * vi;
  r[7] = (-b[0] * b[5] + b[3] * b[2]) * vi;
}

// inter = rec * phys  (row-major rec, region.cc:82-90)
template <typename T>
void to_inter(T* ri, const T* rec, const T* rp) {
  ri[0] = rp[0] * rec[0] + rp[1] * rec[1] + rp[2] * rec[2];
  ri[1] = rp[0] * rec[3] + rp[1] * rec[4] + rp[2] * rec[5];
  ri[2] = rp[0] * rec[6] + rp[1] * rec[7] + rp[2] * rec[8];
}

// phys = box^T * inter  (region.cc:92-101)
template <typename T>
void to_phys(T* rp, const T* box, const T* ri) {
  rp[0] = ri[0] * box[0] + ri[1] * box[3] + ri[2] * box[6];
  rp[1] = ri[0] * box[1] + ri[1] * box[4] + ri[2] * box[7];
  rp[2] = ri[0] * box[2] + ri[1] * box[5] + ri[2] * box[8];
}

// source/lib/src/coord.cc:13-28 normalize_coord_cpu: wrap into [0,1) in
// fractional coordinates, all arithmetic in the coordinate precision.
template <typename T>
void normalize_coord(T* coord, int natom, const T* box) {
  T rec[9];
  rec_box(rec, box);
  for (int ii = 0; ii < natom; ++ii) {
    T ri[3];
    to_inter(ri, rec, coord + 3 * ii);
    for (int dd = 0; dd < 3; ++dd) {
      ri[dd] = std::fmod(ri[dd], static_cast<T>(1.));
      if (ri[dd] < static_cast<T>(0.)) ri[dd] += static_cast<T>(1.);
    }
    to_phys(coord + 3 * ii, box, ri);
  }
}

// ------------------------------------------------------------ ghost copy --
// Cell geometry of source/lib/src/neighbor_list.cc:745-775 (copy_coord) with
// SimulationRegion<double>::toFaceDistance (SimulationRegion_Impl.h:364-372).
struct CellGeom {
  int ncell[3];
  int ngcell[3];
  double to_face[3];
  double box[9];
  double rec[9];
};

void cell_geom(CellGeom& g, const double* box, double rc) {
  std::copy(box, box + 9, g.box);
  rec_box(g.rec, g.box);
  double vol = det3_abs(g.box);
  auto cprod = [](const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  double t[3];
  const int pa[3] = {3, 6, 0}, pb[3] = {6, 0, 3};
  for (int dd = 0; dd < 3; ++dd) {
    cprod(g.box + pa[dd], g.box + pb[dd], t);
    g.to_face[dd] = vol * (1. / std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
  }
  for (int dd = 0; dd < 3; ++dd) {
    g.ncell[dd] = static_cast<int>(g.to_face[dd] / rc);
    if (g.ncell[dd] == 0) g.ncell[dd] = 1;
    double cs = g.to_face[dd] / g.ncell[dd];
    g.ngcell[dd] = static_cast<int>(rc / cs) + 1;
  }
}

// neighbor_list.cc:727-743 compute_pbc_shift
int pbc_shift(int idx, int n) {
  int s = 0;
  if (idx < 0) {
    s = 1;
    while (idx + s * n < 0) ++s;
  } else if (idx >= n) {
    s = -1;
    while (idx + s * n >= n) --s;
  }
  return s;
}

// Local cell of an atom: neighbor_list.cc:86-111 (build_clist) with
// nat_stt = ext_stt = 0, cell size 1/ncell in fractional coordinates.
void local_cell(int* idx, const CellGeom& g, const double* x) {
  double p[3] = {x[0], x[1], x[2]};
  double in[3];
  in[0] = p[0] * g.rec[0] + p[1] * g.rec[1] + p[2] * g.rec[2];
  in[1] = p[0] * g.rec[3] + p[1] * g.rec[4] + p[2] * g.rec[5];
  in[2] = p[0] * g.rec[6] + p[1] * g.rec[7] + p[2] * g.rec[8];
  for (int dd = 0; dd < 3; ++dd) {
    double cs = 1. / g.ncell[dd];
    int k = static_cast<int>(in[dd] / cs);
    if (in[dd] < 0.) --k;
    if (k < 0) k = 0;
    if (k >= g.ncell[dd]) k = g.ncell[dd] - 1;
    idx[dd] = k;
  }
}

// source/lib/src/neighbor_list.cc:745-845 copy_coord, via coord.cc:30-67
// copy_coord_cpu.  Local atoms first, then for every extended cell in
// lexicographic order (x slowest) that is not a local cell, the atoms of its
// periodic source cell in ascending local index, shifted by the image vector.
// Arithmetic in double, result rounded to the coordinate type.
template <typename T>
int copy_coord(std::vector<T>& out_c, std::vector<int>& out_t,
               std::vector<int>& mapping, const T* in_c, const int* in_t,
               int nloc, double rc, const T* box_t) {
  double box[9];
  for (int i = 0; i < 9; ++i) box[i] = box_t[i];
  CellGeom g;
  cell_geom(g, box, rc);
  const int* nc = g.ncell;
  std::vector<std::vector<int>> clist(static_cast<size_t>(nc[0]) * nc[1] * nc[2]);
  std::vector<double> cd(static_cast<size_t>(nloc) * 3);
  for (int i = 0; i < nloc * 3; ++i) cd[i] = in_c[i];
  for (int ii = 0; ii < nloc; ++ii) {
    int idx[3];
    local_cell(idx, g, &cd[ii * 3]);
    clist[(idx[0] * nc[1] + idx[1]) * nc[2] + idx[2]].push_back(ii);
  }
  out_c.assign(in_c, in_c + nloc * 3);
  out_t.assign(in_t, in_t + nloc);
  mapping.resize(nloc);
  for (int i = 0; i < nloc; ++i) mapping[i] = i;
  const int* ng = g.ngcell;
  int ii[3];
  for (ii[0] = -ng[0]; ii[0] < nc[0] + ng[0]; ++ii[0]) {
    int s0 = pbc_shift(ii[0], nc[0]);
    for (ii[1] = -ng[1]; ii[1] < nc[1] + ng[1]; ++ii[1]) {
      int s1 = pbc_shift(ii[1], nc[1]);
      for (ii[2] = -ng[2]; ii[2] < nc[2] + ng[2]; ++ii[2]) {
        int s2 = pbc_shift(ii[2], nc[2]);
        if (ii[0] >= 0 && ii[0] < nc[0] && ii[1] >= 0 && ii[1] < nc[1] &&
            ii[2] >= 0 && ii[2] < nc[2])
          continue;
        double sd[3] = {(double)s0, (double)s1, (double)s2};
        double sv[3];
        sv[0] = sd[0] * box[0] + sd[1] * box[3] + sd[2] * box[6];
        sv[1] = sd[0] * box[1] + sd[1] * box[4] + sd[2] * box[7];
        sv[2] = sd[0] * box[2] + sd[1] * box[5] + sd[2] * box[8];
        int j0 = ii[0] + s0 * nc[0], j1 = ii[1] + s1 * nc[1], j2 = ii[2] + s2 * nc[2];
        const std::vector<int>& cl = clist[(j0 * nc[1] + j1) * nc[2] + j2];
        for (int p : cl) {
          for (int dd = 0; dd < 3; ++dd)
            out_c.push_back(static_cast<T>(cd[p * 3 + dd] - sv[dd]));
          out_t.push_back(in_t[p]);
          mapping.push_back(p);
        }
      }
    }
  }
  return static_cast<int>(out_t.size());
}

// ------------------------------------------------------- neighbour lists --
// source/lib/src/neighbor_list.cc:873-916 build_nlist_cpu: all j != i with
// (c_i - c_j)^2 < rc^2 evaluated in the coordinate type, rc^2 formed in float.
template <typename T>
void build_nlist(std::vector<std::vector<int>>& jlist, const T* c, int nloc,
                 int nall, float rcut) {
  const T rc2 = rcut * rcut;
  jlist.assign(nloc, {});
#pragma omp parallel for schedule(static)
  for (int ii = 0; ii < nloc; ++ii) {
    for (int jj = 0; jj < nall; ++jj) {
      if (jj == ii) continue;
      T d0 = c[ii * 3 + 0] - c[jj * 3 + 0];
      T d1 = c[ii * 3 + 1] - c[jj * 3 + 1];
      T d2 = c[ii * 3 + 2] - c[jj * 3 + 2];
      T r2 = d0 * d0 + d1 * d1 + d2 * d2;
      if (r2 < rc2) jlist[ii].push_back(jj);
    }
  }
}

// The O(N) cell-list candidate build of source/lib/src/neighbor_list.cc:303-420
// (build_nlist with build_clist / build_nlist_cell), on the extended
// coordinates: extended atoms are binned into cells at least rcut (1 + 1e-3)
// wide over their bounding box, and each local atom tests the atoms of its
// own and the 26 adjacent cells with the predicate of build_nlist_cpu
// (r^2 < rc^2 in the coordinate type, diff = c_i - c_j).  Every pair within
// rcut lies in adjacent cells, so the candidate SET equals the brute-force
// build's; the formatting sorts it, so the formatted list is identical.
template <typename T>
void build_nlist_cells(std::vector<std::vector<int>>& jlist, const T* c, int nloc,
                       int nall, float rcut) {
  const T rc2 = rcut * rcut;
  jlist.assign(nloc, {});
  if (nall == 0) return;
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) lo[d] = hi[d] = (double)c[d];
  for (int j = 1; j < nall; ++j)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], (double)c[j * 3 + d]);
      hi[d] = std::max(hi[d], (double)c[j * 3 + d]);
    }
  const double cs = (double)rcut * (1.0 + 1e-3);
  int nc[3];
  for (int d = 0; d < 3; ++d) nc[d] = std::max(1, (int)((hi[d] - lo[d]) / cs));
  auto cell_of = [&](int j, int* k) {
    for (int d = 0; d < 3; ++d) {
      // cells of width (hi - lo) / nc >= cs; the last cell takes the top edge
      int v = (int)(((double)c[j * 3 + d] - lo[d]) / (hi[d] - lo[d] + 1e-300) * nc[d]);
      k[d] = v < 0 ? 0 : (v >= nc[d] ? nc[d] - 1 : v);
    }
  };
  const long ncell = (long)nc[0] * nc[1] * nc[2];
  std::vector<int> start(ncell + 1, 0), order(nall);
  std::vector<int> cell(nall);
  for (int j = 0; j < nall; ++j) {
    int k[3];
    cell_of(j, k);
    cell[j] = (k[0] * nc[1] + k[1]) * nc[2] + k[2];
    ++start[cell[j] + 1];
  }
  for (long q = 0; q < ncell; ++q) start[q + 1] += start[q];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int j = 0; j < nall; ++j) order[fill[cell[j]]++] = j;  // ascending j per cell
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int ii = 0; ii < nloc; ++ii) {
    int k[3];
    cell_of(ii, k);
    std::vector<int>& out = jlist[ii];
    for (int a = std::max(0, k[0] - 1); a <= std::min(nc[0] - 1, k[0] + 1); ++a)
      for (int b = std::max(0, k[1] - 1); b <= std::min(nc[1] - 1, k[1] + 1); ++b)
        for (int e = std::max(0, k[2] - 1); e <= std::min(nc[2] - 1, k[2] + 1); ++e) {
          const long q = ((long)a * nc[1] + b) * nc[2] + e;
          for (int p = start[q]; p < start[q + 1]; ++p) {
            const int jj = order[p];
            if (jj == ii) continue;
            T d0 = c[ii * 3 + 0] - c[jj * 3 + 0];
            T d1 = c[ii * 3 + 1] - c[jj * 3 + 1];
            T d2 = c[ii * 3 + 2] - c[jj * 3 + 2];
            T r2 = d0 * d0 + d1 * d1 + d2 * d2;
            if (r2 < rc2) out.push_back(jj);
          }
        }
    std::sort(out.begin(), out.end());
  }
}

// source/lib/src/fmt_nlist.cc:14-26 (NeighborInfo ordering) and :98-143
// (format_nlist_i_cpu): keep j with float r^2 <= float rc^2 where
// diff = (float)x_j - (float)x_i; order by (type, float r^2, index); fill
// type t into [sec[t], sec[t+1]) and drop the rest (farthest first).
struct NeiKey {
  int type;
  float dist;
  int index;
  bool operator<(const NeiKey& b) const {
    return type < b.type ||
           (type == b.type && (dist < b.dist || (dist == b.dist && index < b.index)));
  }
};

template <typename T>
int format_nlist_i(int* fmt, const T* posi, const int* type, int i_idx,
                   const std::vector<int>& cand, float rcut, const int* sec,
                   int ntypes) {
  const int nnei = sec[ntypes];
  for (int k = 0; k < nnei; ++k) fmt[k] = -1;
  std::vector<NeiKey> sel;
  sel.reserve(cand.size());
  const float rc2 = rcut * rcut;
  for (int j : cand) {
    if (type[j] < 0) continue;
    float d0 = (float)posi[j * 3 + 0] - (float)posi[i_idx * 3 + 0];
    float d1 = (float)posi[j * 3 + 1] - (float)posi[i_idx * 3 + 1];
    float d2 = (float)posi[j * 3 + 2] - (float)posi[i_idx * 3 + 2];
    float r2 = d0 * d0 + d1 * d1 + d2 * d2;
    if (r2 <= rc2) sel.push_back({type[j], r2, j});
  }
  std::sort(sel.begin(), sel.end());
  std::vector<int> it(sec, sec + ntypes);
  int overflowed = -1;
  for (const NeiKey& k : sel) {
    if (it[k.type] < sec[k.type + 1])
      fmt[it[k.type]++] = k.index;
    else
      overflowed = k.type;
  }
  return overflowed;
}

// source/lib/include/switcher.h:60-83 spline5_switch
template <typename T>
void spline5_switch(T& vv, T& dd, T xx, float rmin, float rmax) {
  if (xx < rmin) {
    dd = 0;
    vv = 1;
  } else if (xx < rmax) {
    T uu = (xx - rmin) / (rmax - rmin);
    T du = static_cast<T>(1.) / (rmax - rmin);
    vv = uu * uu * uu * (static_cast<T>(-6.) * uu * uu + static_cast<T>(15.) * uu - static_cast<T>(10.)) +
         static_cast<T>(1.);
    dd = (static_cast<T>(3.) * uu * uu *
              (static_cast<T>(-6.) * uu * uu + static_cast<T>(15.) * uu - static_cast<T>(10.)) +
          uu * uu * uu * (static_cast<T>(-12.) * uu + static_cast<T>(15.))) *
         du;
  } else {
    dd = 0;
    vv = 0;
  }
}

// source/lib/src/env_mat.cc:122-226 env_mat_a_cpu: per neighbour slot the row
// s(r) * [1/r, x/r^2, y/r^2, z/r^2] and its derivative wrt r_ij (12 values).
// A section stops at its first empty slot.
template <typename T>
void env_mat_a_row(T* em, T* dem, T* rij, const T* posi, int i_idx,
                   const int* fmt, const int* sec, int ntypes, float rmin,
                   float rmax) {
  const int nnei = sec[ntypes];
  std::fill(em, em + nnei * 4, T(0));
  std::fill(dem, dem + nnei * 12, T(0));
  std::fill(rij, rij + nnei * 3, T(0));
  for (int s = 0; s < ntypes; ++s) {
    for (int jj = sec[s]; jj < sec[s + 1]; ++jj) {
      int j = fmt[jj];
      if (j < 0) break;
      T* rr = rij + jj * 3;
      for (int dd = 0; dd < 3; ++dd) rr[dd] = posi[j * 3 + dd] - posi[i_idx * 3 + dd];
      T nr2 = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
      // env_mat.cc calls the C library's sqrt(double) unqualified, so a float
      // r^2 is promoted and 1/sqrt is formed in double before rounding.
      T inr = static_cast<T>(static_cast<T>(1.) / std::sqrt(static_cast<double>(nr2)));
      T nr = nr2 * inr;
      T inr2 = inr * inr;
      T inr4 = inr2 * inr2;
      T inr3 = inr4 * nr;
      T sw, dsw;
      spline5_switch(sw, dsw, nr, rmin, rmax);
      T* e = em + jj * 4;
      T* d = dem + jj * 12;
      e[0] = static_cast<T>(1.) / nr;
      e[1] = rr[0] / nr2;
      e[2] = rr[1] / nr2;
      e[3] = rr[2] / nr2;
      for (int dd = 0; dd < 3; ++dd)
        d[dd] = rr[dd] * inr3 * sw - e[0] * dsw * rr[dd] * inr;
      for (int c = 0; c < 3; ++c) {
        for (int dd = 0; dd < 3; ++dd) {
          T t = static_cast<T>(2.) * rr[c] * rr[dd] * inr4;
          if (c == dd) t = t - inr2;
          d[3 + c * 3 + dd] = t * sw - e[1 + c] * dsw * rr[dd] * inr;
        }
      }
      for (int c = 0; c < 4; ++c) e[c] *= sw;
    }
  }
}

// source/lib/src/prod_env_mat.cc:14-108 prod_env_mat_a_cpu: format, env
// row, then (row - avg[t_i]) / std[t_i]; derivative / std.
template <typename T>
void prod_env_mat_a(T* em, T* em_deriv, T* rij, int* nlist, const T* coord,
                    const int* type, const std::vector<std::vector<int>>& cand,
                    const T* avg, const T* std_, int nloc, float rcut,
                    float rcut_smth, const int* sec, int ntypes) {
  const int nnei = sec[ntypes];
  const int nem = nnei * 4;
#pragma omp parallel for schedule(dynamic, 4)
  for (int ii = 0; ii < nloc; ++ii) {
    std::vector<int> fmt(nnei);
    format_nlist_i(fmt.data(), coord, type, ii, cand[ii], rcut, sec, ntypes);
    std::vector<T> e(nem), d(nem * 3), r(nnei * 3);
    env_mat_a_row(e.data(), d.data(), r.data(), coord, ii, fmt.data(), sec, ntypes,
                  rcut_smth, rcut);
    const int t = type[ii];
    for (int jj = 0; jj < nem; ++jj)
      em[(size_t)ii * nem + jj] =
          t >= 0 ? (e[jj] - avg[t * nem + jj]) / std_[t * nem + jj] : T(0);
    for (int jj = 0; jj < nem * 3; ++jj)
      em_deriv[(size_t)ii * nem * 3 + jj] = t >= 0 ? d[jj] / std_[t * nem + jj / 3] : T(0);
    for (int jj = 0; jj < nnei * 3; ++jj) rij[(size_t)ii * nnei * 3 + jj] = r[jj];
    for (int jj = 0; jj < nnei; ++jj) nlist[(size_t)ii * nnei + jj] = fmt[jj];
  }
}

// ------------------------------------------------------------ tabulation --
// source/lib/src/tabulate.cc:19-42 locate_xx: two uniform strides then clamp.
template <typename T>
void locate_xx(T lower, T upper, T mx, T stride0, T stride1, T& xx, int& idx) {
  if (xx < lower) {
    idx = 0;
    xx = 0;
  } else if (xx < upper) {
    idx = (int)((xx - lower) / stride0);
    xx -= (idx * stride0 + lower);
  } else if (xx < mx) {
    int first = int((upper - lower) / stride0);
    idx = first + (int)((xx - upper) / stride1);
    xx -= ((idx - first) * stride1 + upper);
  } else {
    idx = int((upper - lower) / stride0) + (int)((mx - upper) / stride1) - 1;
    xx = 0;
  }
}

// The padding fold of tabulate.cc:108-155: with is_sorted, the first slot
// whose x equals the last slot's x and whose em[1:4] are all zero stands for
// itself and every later slot, so it is weighted (nnei - j) and the loop ends.
template <typename T>
bool is_fold_point(const T* em_row, T x, T last_x) {
  return last_x == x && em_row[1] == 0. && em_row[2] == 0. && em_row[3] == 0.;
}

// source/lib/src/tabulate.cc:80-157 tabulate_fusion_se_a_cpu
template <typename T>
void tabulate_fwd(T* out, const T* table, const T* info, const T* em_x,
                  const T* em, int nloc, int nnei, int M) {
  const T lo = info[0], up = info[1], mx = info[2], s0 = info[3], s1 = info[4];
#pragma omp parallel for schedule(static)
  for (int ii = 0; ii < nloc; ++ii) {
    T* o = out + (size_t)ii * 4 * M;
    std::fill(o, o + 4 * M, T(0));
    const T last = em_x[(size_t)ii * nnei + nnei - 1];
    for (int jj = 0; jj < nnei; ++jj) {
      const T* ll = em + ((size_t)ii * nnei + jj) * 4;
      T xx = em_x[(size_t)ii * nnei + jj];
      bool fold = is_fold_point(ll, xx, last);
      int idx = 0;
      locate_xx(lo, up, mx, s0, s1, xx, idx);
      const T w = fold ? T(nnei - jj) : T(1);
      for (int k = 0; k < M; ++k) {
        const T* a = table + (size_t)idx * M * 6 + 6 * k;
        T v = a[0] + (a[1] + (a[2] + (a[3] + (a[4] + a[5] * xx) * xx) * xx) * xx) * xx;
        for (int m = 0; m < 4; ++m) o[m * M + k] += w * v * ll[m];
      }
      if (fold) break;
    }
  }
}

// source/lib/src/tabulate.cc:158-260 tabulate_fusion_se_a_grad_cpu
template <typename T>
void tabulate_grad(T* dy_dem_x, T* dy_dem, const T* table, const T* info,
                   const T* em_x, const T* em, const T* dy, int nloc, int nnei,
                   int M) {
  const T lo = info[0], up = info[1], mx = info[2], s0 = info[3], s1 = info[4];
#pragma omp parallel for schedule(static)
  for (int ii = 0; ii < nloc; ++ii) {
    std::fill(dy_dem_x + (size_t)ii * nnei, dy_dem_x + (size_t)(ii + 1) * nnei, T(0));
    std::fill(dy_dem + (size_t)ii * nnei * 4, dy_dem + (size_t)(ii + 1) * nnei * 4, T(0));
    const T last = em_x[(size_t)ii * nnei + nnei - 1];
    const T* g = dy + (size_t)ii * 4 * M;
    for (int jj = 0; jj < nnei; ++jj) {
      const T* ll = em + ((size_t)ii * nnei + jj) * 4;
      T xx = em_x[(size_t)ii * nnei + jj];
      bool fold = is_fold_point(ll, xx, last);
      int idx = 0;
      locate_xx(lo, up, mx, s0, s1, xx, idx);
      const T w = fold ? T(nnei - jj) : T(1);
      T gx = 0;
      T* dm = dy_dem + ((size_t)ii * nnei + jj) * 4;
      for (int k = 0; k < M; ++k) {
        const T* a = table + (size_t)idx * M * 6 + 6 * k;
        T v = a[0] + (a[1] + (a[2] + (a[3] + (a[4] + a[5] * xx) * xx) * xx) * xx) * xx;
        T dv = a[1] + (2 * a[2] + (3 * a[3] + (4 * a[4] + 5 * a[5] * xx) * xx) * xx) * xx;
        T r0 = g[0 * M + k], r1 = g[1 * M + k], r2 = g[2 * M + k], r3 = g[3 * M + k];
        T dot = ll[0] * r0 + ll[1] * r1 + ll[2] * r2 + ll[3] * r3;
        // tabulate.cc:228-239 multiplies the fold weight last.
        gx += fold ? dv * dot * w : dv * dot;
        dm[0] += fold ? v * r0 * w : v * r0;
        dm[1] += fold ? v * r1 * w : v * r1;
        dm[2] += fold ? v * r2 * w : v * r2;
        dm[3] += fold ? v * r3 * w : v * r3;
      }
      dy_dem_x[(size_t)ii * nnei + jj] = gx;
      if (fold) break;
    }
  }
}

// source/lib/src/tabulate.cc:261-384 tabulate_fusion_se_a_grad_grad_cpu
template <typename T>
void tabulate_grad_grad(T* dz_dy, const T* table, const T* info, const T* em_x,
                        const T* em, const T* dz_dem_x, const T* dz_dem,
                        int nloc, int nnei, int M) {
  const T lo = info[0], up = info[1], mx = info[2], s0 = info[3], s1 = info[4];
#pragma omp parallel for schedule(static)
  for (int ii = 0; ii < nloc; ++ii) {
    T* o = dz_dy + (size_t)ii * 4 * M;
    std::fill(o, o + 4 * M, T(0));
    const T last = em_x[(size_t)ii * nnei + nnei - 1];
    for (int jj = 0; jj < nnei; ++jj) {
      const T* ll = em + ((size_t)ii * nnei + jj) * 4;
      const T* hh = dz_dem + ((size_t)ii * nnei + jj) * 4;
      T xx = em_x[(size_t)ii * nnei + jj];
      T dzx = dz_dem_x[(size_t)ii * nnei + jj];
      bool fold = is_fold_point(ll, xx, last);
      int idx = 0;
      locate_xx(lo, up, mx, s0, s1, xx, idx);
      const T w = fold ? T(nnei - jj) : T(1);
      for (int k = 0; k < M; ++k) {
        const T* a = table + (size_t)idx * M * 6 + 6 * k;
        T v = a[0] + (a[1] + (a[2] + (a[3] + (a[4] + a[5] * xx) * xx) * xx) * xx) * xx;
        T dv = a[1] + (2 * a[2] + (3 * a[3] + (4 * a[4] + 5 * a[5] * xx) * xx) * xx) * xx;
        for (int m = 0; m < 4; ++m) o[m * M + k] += w * (v * hh[m] + dzx * dv * ll[m]);
      }
      if (fold) break;
    }
  }
}

// ------------------------------------------------------ force and virial --
// source/lib/src/prod_force.cc:22-72 prod_force_a_cpu (nframes of nloc
// centres, force laid out [nframes, nall, 3]).
template <typename T>
void prod_force_a(T* force, const T* net_deriv, const T* env_deriv,
                  const int* nlist, int nloc, int nall, int nnei, int nframes) {
  const int nd = 4 * nnei;
  std::memset(force, 0, sizeof(T) * (size_t)nframes * nall * 3);
  for (int f = 0; f < nframes; ++f) {
    T* F = force + (size_t)f * nall * 3;
    for (int ii = 0; ii < nloc; ++ii) {
      const size_t i = (size_t)f * nloc + ii;
      const T* g = net_deriv + i * nd;
      const T* d = env_deriv + i * nd * 3;
      for (int aa = 0; aa < nd; ++aa)
        for (int dd = 0; dd < 3; ++dd) F[ii * 3 + dd] -= g[aa] * d[aa * 3 + dd];
      for (int jj = 0; jj < nnei; ++jj) {
        int j = nlist[i * nnei + jj];
        if (j < 0) continue;
        for (int aa = jj * 4; aa < jj * 4 + 4; ++aa)
          for (int dd = 0; dd < 3; ++dd) F[j * 3 + dd] += g[aa] * d[aa * 3 + dd];
      }
    }
  }
}

// source/lib/src/prod_virial.cc:22-68 prod_virial_a_cpu (one frame).
template <typename T>
void prod_virial_a(T* virial, T* atom_virial, const T* net_deriv,
                   const T* env_deriv, const T* rij, const int* nlist, int nloc,
                   int nall, int nnei) {
  const int nd = 4 * nnei;
  for (int k = 0; k < 9; ++k) virial[k] = 0;
  std::memset(atom_virial, 0, sizeof(T) * (size_t)nall * 9);
  for (int ii = 0; ii < nloc; ++ii) {
    for (int jj = 0; jj < nnei; ++jj) {
      int j = nlist[(size_t)ii * nnei + jj];
      if (j < 0) continue;
      for (int aa = jj * 4; aa < jj * 4 + 4; ++aa) {
        T pref = static_cast<T>(-1.0) * net_deriv[(size_t)ii * nd + aa];
        for (int d0 = 0; d0 < 3; ++d0)
          for (int d1 = 0; d1 < 3; ++d1) {
            T v = pref * rij[((size_t)ii * nnei + jj) * 3 + d1] *
                  env_deriv[((size_t)ii * nd + aa) * 3 + d0];
            virial[d0 * 3 + d1] -= v;
            atom_virial[(size_t)j * 9 + d0 * 3 + d1] -= v;
          }
      }
    }
  }
}

// source/lib/src/prod_force_grad.cc:22-73 prod_force_grad_a_cpu
template <typename T>
void prod_force_grad_a(T* grad_net, const T* grad, const T* env_deriv,
                       const int* nlist, int nloc, int nnei, int nframes) {
  const int nd = 4 * nnei;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nframes * nloc; ++i) {
    T* gn = grad_net + (size_t)i * nd;
    const T* d = env_deriv + (size_t)i * nd * 3;
    for (int aa = 0; aa < nd; ++aa) {
      gn[aa] = 0;
      for (int dd = 0; dd < 3; ++dd) gn[aa] -= grad[(size_t)i * 3 + dd] * d[aa * 3 + dd];
    }
    const int f = i / nloc;
    for (int jj = 0; jj < nnei; ++jj) {
      int j = nlist[(size_t)i * nnei + jj];
      if (j >= nloc) j = j % nloc;
      if (j < 0) continue;
      for (int aa = jj * 4; aa < jj * 4 + 4; ++aa)
        for (int dd = 0; dd < 3; ++dd)
          gn[aa] += grad[((size_t)f * nloc + j) * 3 + dd] * d[aa * 3 + dd];
    }
  }
}

// source/lib/src/prod_virial_grad.cc:20-66 prod_virial_grad_a_cpu (one frame)
template <typename T>
void prod_virial_grad_a(T* grad_net, const T* grad, const T* env_deriv,
                        const T* rij, const int* nlist, int nloc, int nnei) {
  const int nd = 4 * nnei;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nloc; ++i) {
    T* gn = grad_net + (size_t)i * nd;
    for (int aa = 0; aa < nd; ++aa) gn[aa] = 0;
    for (int jj = 0; jj < nnei; ++jj) {
      int j = nlist[(size_t)i * nnei + jj];
      if (j < 0) continue;
      for (int aa = jj * 4; aa < jj * 4 + 4; ++aa)
        for (int d0 = 0; d0 < 3; ++d0)
          for (int d1 = 0; d1 < 3; ++d1)
            // prod_virial_grad.cc:56-59 uses the double literal -1.0, so the
            // product and the update are formed in double.
            gn[aa] = static_cast<T>(static_cast<double>(gn[aa]) -
                                    -1.0 * grad[d0 * 3 + d1] *
                                        rij[((size_t)i * nnei + jj) * 3 + d1] *
                                        env_deriv[((size_t)i * nd + aa) * 3 + d0]);
    }
  }
}

// The whole TF ProdEnvMatA op for one frame in the internal-PBC mode
// (source/op/tf/prod_env_mat_multi_device.cc:417-438 nei_mode 1, :1309-1372,
// :590-622): normalise, copy ghosts, brute-force candidates, format + env
// mat, then map neighbour indices back to local atoms.
template <typename T>
int prod_env_mat_a_pbc(T* em, T* em_deriv, T* rij, int* nlist, const T* coord,
                       const int* type, const T* box, const T* avg,
                       const T* std_, int nloc, float rcut, float rcut_smth,
                       const int* sec, int ntypes, int map_to_local,
                       int* nall_out, T* ext_coord, int* ext_type,
                       int* ext_map, int ext_cap, int cell_list = 0) {
  std::vector<T> c(coord, coord + (size_t)nloc * 3);
  normalize_coord(c.data(), nloc, box);
  std::vector<T> cc;
  std::vector<int> ct, map;
  int nall = copy_coord(cc, ct, map, c.data(), type, nloc, rcut, box);
  if (nall_out) *nall_out = nall;
  if (ext_coord && nall <= ext_cap) {
    std::copy(cc.begin(), cc.end(), ext_coord);
    std::copy(ct.begin(), ct.end(), ext_type);
    std::copy(map.begin(), map.end(), ext_map);
  }
  std::vector<std::vector<int>> cand;
  if (cell_list)
    build_nlist_cells(cand, cc.data(), nloc, nall, rcut);
  else
    build_nlist(cand, cc.data(), nloc, nall, rcut);
  prod_env_mat_a(em, em_deriv, rij, nlist, cc.data(), ct.data(), cand, avg, std_,
                 nloc, rcut, rcut_smth, sec, ntypes);
  const int nnei = sec[ntypes];
  if (map_to_local)
    for (size_t k = 0; k < (size_t)nloc * nnei; ++k)
      if (nlist[k] >= 0) nlist[k] = map[nlist[k]];
  return 0;
}

// ------------------------------------------------- forward_lower path --
// Neighbour-list formatting of the PyTorch forward_lower path for a
// compressed se_e2_a (need_sorted_nlist_for_lower: extra_nlist_sort):
// deepmd/pt/model/model/make_model.py:541-598 (_format_nlist) then
// deepmd/pt/utils/nlist.py:304-337 (nlist_distinguish_types).  Per local atom
// i (the first nloc extended atoms): every listed j >= 0 at distance
// rr = |x_i - x_j| (formed in T, as torch.linalg.norm), sorted ascending
// (ties by list position); rr > rcut dropped; the nearest nnei kept; then,
// in that order, the first sel[t] of type t fill section t.
template <typename T>
void format_nlist_pt(int* out, const T* ext, const int* etype, const int* nl_in, int nloc,
                     int nnei_in, T rcut, const int* sec, int ntypes) {
  const int nnei = sec[ntypes];
#pragma omp parallel for schedule(dynamic, 8)
  for (int i = 0; i < nloc; ++i) {
    std::vector<std::pair<T, int>> c;
    for (int p = 0; p < nnei_in; ++p) {
      const int j = nl_in[(size_t)i * nnei_in + p];
      if (j < 0) continue;
      T d0 = ext[i * 3] - ext[j * 3], d1 = ext[i * 3 + 1] - ext[j * 3 + 1],
        d2 = ext[i * 3 + 2] - ext[j * 3 + 2];
      T rr = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
      if (!(rr > rcut)) c.push_back({rr, p});
    }
    std::sort(c.begin(), c.end());
    if ((int)c.size() > nnei) c.resize(nnei);
    int* o = out + (size_t)i * nnei;
    std::fill(o, o + nnei, -1);
    std::vector<int> fill(ntypes, 0);
    for (const auto& e : c) {
      const int j = nl_in[(size_t)i * nnei_in + e.second];
      const int t = etype[j];
      if (t < 0 || t >= ntypes) continue;
      if (fill[t] < sec[t + 1] - sec[t]) o[sec[t] + fill[t]++] = j;
    }
  }
}

// env rows for an already formatted list (env_mat_a_cpu rows as above,
// prod_env_mat.cc:84-100 normalisation by the centre atom's type)
template <typename T>
void env_mat_a_nlist(T* em, T* em_deriv, T* rij, const T* ext, const int* etype,
                     const int* fmt, const T* avg, const T* std_, int nloc, float rcut,
                     float rcut_smth, const int* sec, int ntypes) {
  const int nnei = sec[ntypes];
  const int nem = nnei * 4;
#pragma omp parallel for schedule(dynamic, 8)
  for (int ii = 0; ii < nloc; ++ii) {
    std::vector<T> e(nem), d(nem * 3), r(nnei * 3);
    env_mat_a_row(e.data(), d.data(), r.data(), ext, ii, fmt + (size_t)ii * nnei, sec, ntypes,
                  rcut_smth, rcut);
    const int t = etype[ii];
    for (int jj = 0; jj < nem; ++jj)
      em[(size_t)ii * nem + jj] =
          t >= 0 ? (e[jj] - avg[t * nem + jj]) / std_[t * nem + jj] : T(0);
    for (int jj = 0; jj < nem * 3; ++jj)
      em_deriv[(size_t)ii * nem * 3 + jj] = t >= 0 ? d[jj] / std_[t * nem + jj / 3] : T(0);
    for (int jj = 0; jj < nnei * 3; ++jj) rij[(size_t)ii * nnei * 3 + jj] = r[jj];
  }
}

}  // namespace

// ------------------------------------------------------------- C entry --
#define OR_EXPORT extern "C" __attribute__((visibility("default")))

#define OR_INSTANTIATE(T, SFX)                                                 \
  OR_EXPORT void or_normalize_coord_##SFX(T* coord, int natom, const T* box) { \
    normalize_coord(coord, natom, box);                                        \
  }                                                                            \
  OR_EXPORT int or_copy_coord_##SFX(T* out_c, int* out_t, int* mapping,        \
                                    int cap, const T* in_c, const int* in_t,   \
                                    int nloc, float rcut, const T* box) {      \
    std::vector<T> c;                                                          \
    std::vector<int> t, m;                                                     \
    int nall = copy_coord(c, t, m, in_c, in_t, nloc, rcut, box);               \
    if (nall <= cap) {                                                         \
      std::copy(c.begin(), c.end(), out_c);                                    \
      std::copy(t.begin(), t.end(), out_t);                                    \
      std::copy(m.begin(), m.end(), mapping);                                  \
    }                                                                          \
    return nall;                                                               \
  }                                                                            \
  OR_EXPORT void or_format_nlist_##SFX(int* nlist, const T* coord,             \
                                       const int* type, int nloc, int nall,    \
                                       float rcut, const int* sec,             \
                                       int ntypes) {                           \
    std::vector<std::vector<int>> cand;                                        \
    build_nlist(cand, coord, nloc, nall, rcut);                                \
    const int nnei = sec[ntypes];                                              \
    _Pragma("omp parallel for schedule(dynamic, 8)") for (int i = 0; i < nloc; \
                                                          ++i)                 \
        format_nlist_i(nlist + (size_t)i * nnei, coord, type, i, cand[i],      \
                       rcut, sec, ntypes);                                     \
  }                                                                            \
  OR_EXPORT void or_prod_env_mat_a_##SFX(                                      \
      T* em, T* em_deriv, T* rij, int* nlist, const T* coord, const int* type, \
      const T* avg, const T* std_, int nloc, int nall, float rcut,             \
      float rcut_smth, const int* sec, int ntypes) {                           \
    std::vector<std::vector<int>> cand;                                        \
    build_nlist(cand, coord, nloc, nall, rcut);                                \
    prod_env_mat_a(em, em_deriv, rij, nlist, coord, type, cand, avg, std_,     \
                   nloc, rcut, rcut_smth, sec, ntypes);                        \
  }                                                                            \
  OR_EXPORT int or_prod_env_mat_a_pbc_##SFX(                                   \
      T* em, T* em_deriv, T* rij, int* nlist, const T* coord, const int* type, \
      const T* box, const T* avg, const T* std_, int nloc, float rcut,         \
      float rcut_smth, const int* sec, int ntypes, int map_to_local,           \
      int* nall_out, T* ext_coord, int* ext_type, int* ext_map,                \
      int ext_cap) {                                                           \
    return prod_env_mat_a_pbc(em, em_deriv, rij, nlist, coord, type, box, avg, \
                              std_, nloc, rcut, rcut_smth, sec, ntypes,        \
                              map_to_local, nall_out, ext_coord, ext_type,     \
                              ext_map, ext_cap);                               \
  }                                                                            \
  OR_EXPORT int or_prod_env_mat_a_pbc_cells_##SFX(                             \
      T* em, T* em_deriv, T* rij, int* nlist, const T* coord, const int* type, \
      const T* box, const T* avg, const T* std_, int nloc, float rcut,         \
      float rcut_smth, const int* sec, int ntypes, int map_to_local,           \
      int* nall_out, T* ext_coord, int* ext_type, int* ext_map,                \
      int ext_cap) {                                                           \
    return prod_env_mat_a_pbc(em, em_deriv, rij, nlist, coord, type, box, avg, \
                              std_, nloc, rcut, rcut_smth, sec, ntypes,        \
                              map_to_local, nall_out, ext_coord, ext_type,     \
                              ext_map, ext_cap, 1);                            \
  }                                                                            \
  OR_EXPORT void or_format_nlist_pt_##SFX(int* out, const T* ext,              \
                                          const int* etype, const int* nl_in,  \
                                          int nloc, int nnei_in, double rcut,  \
                                          const int* sec, int ntypes) {        \
    format_nlist_pt(out, ext, etype, nl_in, nloc, nnei_in, (T)rcut, sec,       \
                    ntypes);                                                   \
  }                                                                            \
  OR_EXPORT void or_env_mat_a_nlist_##SFX(                                     \
      T* em, T* em_deriv, T* rij, const T* ext, const int* etype,              \
      const int* fmt, const T* avg, const T* std_, int nloc, float rcut,       \
      float rcut_smth, const int* sec, int ntypes) {                           \
    env_mat_a_nlist(em, em_deriv, rij, ext, etype, fmt, avg, std_, nloc, rcut, \
                    rcut_smth, sec, ntypes);                                   \
  }                                                                            \
  OR_EXPORT void or_tabulate_fusion_se_a_##SFX(                                \
      T* out, const T* table, const T* info, const T* em_x, const T* em,       \
      int nloc, int nnei, int M) {                                             \
    tabulate_fwd(out, table, info, em_x, em, nloc, nnei, M);                   \
  }                                                                            \
  OR_EXPORT void or_tabulate_fusion_se_a_grad_##SFX(                           \
      T* dy_dem_x, T* dy_dem, const T* table, const T* info, const T* em_x,    \
      const T* em, const T* dy, int nloc, int nnei, int M) {                   \
    tabulate_grad(dy_dem_x, dy_dem, table, info, em_x, em, dy, nloc, nnei, M); \
  }                                                                            \
  OR_EXPORT void or_tabulate_fusion_se_a_grad_grad_##SFX(                      \
      T* dz_dy, const T* table, const T* info, const T* em_x, const T* em,     \
      const T* dz_dem_x, const T* dz_dem, int nloc, int nnei, int M) {         \
    tabulate_grad_grad(dz_dy, table, info, em_x, em, dz_dem_x, dz_dem, nloc,   \
                       nnei, M);                                               \
  }                                                                            \
  OR_EXPORT void or_prod_force_a_##SFX(T* force, const T* net_deriv,           \
                                       const T* env_deriv, const int* nlist,   \
                                       int nloc, int nall, int nnei,           \
                                       int nframes) {                          \
    prod_force_a(force, net_deriv, env_deriv, nlist, nloc, nall, nnei,         \
                 nframes);                                                     \
  }                                                                            \
  OR_EXPORT void or_prod_virial_a_##SFX(                                       \
      T* virial, T* atom_virial, const T* net_deriv, const T* env_deriv,       \
      const T* rij, const int* nlist, int nloc, int nall, int nnei) {          \
    prod_virial_a(virial, atom_virial, net_deriv, env_deriv, rij, nlist, nloc, \
                  nall, nnei);                                                 \
  }                                                                            \
  OR_EXPORT void or_prod_force_grad_a_##SFX(                                   \
      T* grad_net, const T* grad, const T* env_deriv, const int* nlist,        \
      int nloc, int nnei, int nframes) {                                       \
    prod_force_grad_a(grad_net, grad, env_deriv, nlist, nloc, nnei, nframes);  \
  }                                                                            \
  OR_EXPORT void or_prod_virial_grad_a_##SFX(                                  \
      T* grad_net, const T* grad, const T* env_deriv, const T* rij,            \
      const int* nlist, int nloc, int nnei) {                                  \
    prod_virial_grad_a(grad_net, grad, env_deriv, rij, nlist, nloc, nnei);     \
  }

OR_INSTANTIATE(double, f64)
OR_INSTANTIATE(float, f32)

OR_EXPORT int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
