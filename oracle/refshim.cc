// Test infrastructure only.  extern "C" entry points over the reference's own
// CPU library (source/lib/src/*.cc), compiled from the reference sources by
// oracle/Makefile into oracle/_ref/libref_cpu.so.  The tests use it to check
// the oracle restatement (oracle/oracle.cc) and to generate fixtures; nothing
// in the product links it.  The call sequence of ref_prod_env_mat_a_pbc_* is
// the TF ProdEnvMatA op's internal-PBC mode
// (source/op/tf/prod_env_mat_multi_device.cc:1309-1372 and :590-622).

#include <vector>

#include "coord.h"
#include "fmt_nlist.h"
#include "neighbor_list.h"
#include "prod_env_mat.h"
#include "prod_force.h"
#include "prod_force_grad.h"
#include "prod_virial.h"
#include "prod_virial_grad.h"
#include "region.h"
#include "tabulate.h"

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

template <typename T>
int pbc_env(T* em, T* em_deriv, T* rij, int* nlist, const T* coord,
            const int* type, const T* box, const T* avg, const T* std_,
            int nloc, float rcut, float rcut_smth, const int* sec, int ntypes,
            int map_to_local, int* nall_out, T* ext_coord, int* ext_type,
            int* ext_map, int ext_cap) {
  std::vector<T> c(coord, coord + (size_t)nloc * 3);
  deepmd::Region<T> region;
  deepmd::init_region_cpu(region, box);
  deepmd::normalize_coord_cpu(c.data(), nloc, region);
  int mem = nloc * 64 + 1024, nall = 0;
  std::vector<T> cc;
  std::vector<int> ct, map;
  for (int trial = 0; trial < 20; ++trial) {
    cc.resize((size_t)mem * 3);
    ct.resize(mem);
    map.resize(mem);
    if (deepmd::copy_coord_cpu(cc.data(), ct.data(), map.data(), &nall, c.data(),
                               type, nloc, mem, rcut, region) == 0)
      break;
    mem *= 2;
  }
  if (nall_out) *nall_out = nall;
  if (ext_coord && nall <= ext_cap) {
    std::copy(cc.begin(), cc.begin() + (size_t)nall * 3, ext_coord);
    std::copy(ct.begin(), ct.begin() + nall, ext_type);
    std::copy(map.begin(), map.begin() + nall, ext_map);
  }
  int mem_nnei = 256, max_nnei = 0;
  std::vector<int> ilist(nloc), numneigh(nloc);
  std::vector<int*> firstneigh(nloc);
  std::vector<std::vector<int>> jlist(nloc);
  for (int trial = 0; trial < 20; ++trial) {
    for (int ii = 0; ii < nloc; ++ii) {
      jlist[ii].resize(mem_nnei);
      firstneigh[ii] = jlist[ii].data();
    }
    deepmd::InputNlist inl(nloc, ilist.data(), numneigh.data(), firstneigh.data());
    if (deepmd::build_nlist_cpu(inl, &max_nnei, cc.data(), nloc, nall, mem_nnei,
                                rcut) == 0)
      break;
    mem_nnei *= 2;
  }
  deepmd::InputNlist inl(nloc, ilist.data(), numneigh.data(), firstneigh.data());
  std::vector<int> secv(sec, sec + ntypes + 1);
  deepmd::prod_env_mat_a_cpu(em, em_deriv, rij, nlist, cc.data(), ct.data(), inl,
                             max_nnei, avg, std_, nloc, nall, rcut, rcut_smth,
                             secv);
  const int nnei = sec[ntypes];
  if (map_to_local)
    for (size_t k = 0; k < (size_t)nloc * nnei; ++k)
      if (nlist[k] >= 0) nlist[k] = map[nlist[k]];
  return 0;
}

template <typename T>
void fmt_nlist(int* nlist, const T* coord, const int* type, int nloc, int nall,
               float rcut, const int* sec, int ntypes) {
  int mem_nnei = 256, max_nnei = 0;
  std::vector<int> ilist(nloc), numneigh(nloc);
  std::vector<int*> firstneigh(nloc);
  std::vector<std::vector<int>> jlist(nloc);
  for (int trial = 0; trial < 20; ++trial) {
    for (int ii = 0; ii < nloc; ++ii) {
      jlist[ii].resize(mem_nnei);
      firstneigh[ii] = jlist[ii].data();
    }
    deepmd::InputNlist inl(nloc, ilist.data(), numneigh.data(), firstneigh.data());
    if (deepmd::build_nlist_cpu(inl, &max_nnei, coord, nloc, nall, mem_nnei,
                                rcut) == 0)
      break;
    mem_nnei *= 2;
  }
  deepmd::InputNlist inl(nloc, ilist.data(), numneigh.data(), firstneigh.data());
  std::vector<int> secv(sec, sec + ntypes + 1);
  deepmd::format_nlist_cpu(nlist, inl, coord, type, nloc, nall, rcut, secv);
}

}  // namespace

#define REF_INSTANTIATE(T, SFX)                                                \
  REF_EXPORT void ref_normalize_coord_##SFX(T* coord, int natom,               \
                                            const T* box) {                    \
    deepmd::Region<T> region;                                                  \
    deepmd::init_region_cpu(region, box);                                      \
    deepmd::normalize_coord_cpu(coord, natom, region);                         \
  }                                                                            \
  REF_EXPORT int ref_copy_coord_##SFX(T* out_c, int* out_t, int* mapping,      \
                                      int cap, const T* in_c, const int* in_t, \
                                      int nloc, float rcut, const T* box) {    \
    deepmd::Region<T> region;                                                  \
    deepmd::init_region_cpu(region, box);                                      \
    int nall = 0;                                                              \
    deepmd::copy_coord_cpu(out_c, out_t, mapping, &nall, in_c, in_t, nloc,     \
                           cap, rcut, region);                                 \
    return nall;                                                               \
  }                                                                            \
  REF_EXPORT int ref_prod_env_mat_a_pbc_##SFX(                                 \
      T* em, T* em_deriv, T* rij, int* nlist, const T* coord, const int* type, \
      const T* box, const T* avg, const T* std_, int nloc, float rcut,         \
      float rcut_smth, const int* sec, int ntypes, int map_to_local,           \
      int* nall_out, T* ext_coord, int* ext_type, int* ext_map,                \
      int ext_cap) {                                                           \
    return pbc_env(em, em_deriv, rij, nlist, coord, type, box, avg, std_,      \
                   nloc, rcut, rcut_smth, sec, ntypes, map_to_local, nall_out, \
                   ext_coord, ext_type, ext_map, ext_cap);                     \
  }                                                                            \
  REF_EXPORT void ref_format_nlist_##SFX(int* nlist, const T* coord,           \
                                         const int* type, int nloc, int nall,  \
                                         float rcut, const int* sec,           \
                                         int ntypes) {                         \
    fmt_nlist(nlist, coord, type, nloc, nall, rcut, sec, ntypes);              \
  }                                                                            \
  REF_EXPORT void ref_tabulate_fusion_se_a_##SFX(                              \
      T* out, const T* table, const T* info, const T* em_x, const T* em,       \
      int nloc, int nnei, int M) {                                             \
    deepmd::tabulate_fusion_se_a_cpu(out, table, info, em_x, em, (const T*)0,  \
                                     nloc, nnei, M);                           \
  }                                                                            \
  REF_EXPORT void ref_tabulate_fusion_se_a_grad_##SFX(                         \
      T* dy_dem_x, T* dy_dem, const T* table, const T* info, const T* em_x,    \
      const T* em, const T* dy, int nloc, int nnei, int M) {                   \
    deepmd::tabulate_fusion_se_a_grad_cpu(dy_dem_x, dy_dem, (T*)0, table,      \
                                          info, em_x, em, (const T*)0, dy,     \
                                          nloc, nnei, M);                      \
  }                                                                            \
  REF_EXPORT void ref_tabulate_fusion_se_a_grad_grad_##SFX(                    \
      T* dz_dy, const T* table, const T* info, const T* em_x, const T* em,     \
      const T* dz_dem_x, const T* dz_dem, int nloc, int nnei, int M) {         \
    deepmd::tabulate_fusion_se_a_grad_grad_cpu(dz_dy, table, info, em_x, em,   \
                                               (const T*)0, dz_dem_x, dz_dem,  \
                                               (const T*)0, nloc, nnei, M);    \
  }                                                                            \
  REF_EXPORT void ref_prod_force_a_##SFX(T* force, const T* net_deriv,         \
                                         const T* env_deriv, const int* nlist, \
                                         int nloc, int nall, int nnei,         \
                                         int nframes) {                        \
    deepmd::prod_force_a_cpu(force, net_deriv, env_deriv, nlist, nloc, nall,   \
                             nnei, nframes);                                   \
  }                                                                            \
  REF_EXPORT void ref_prod_virial_a_##SFX(                                     \
      T* virial, T* atom_virial, const T* net_deriv, const T* env_deriv,       \
      const T* rij, const int* nlist, int nloc, int nall, int nnei) {          \
    deepmd::prod_virial_a_cpu(virial, atom_virial, net_deriv, env_deriv, rij,  \
                              nlist, nloc, nall, nnei);                        \
  }                                                                            \
  REF_EXPORT void ref_prod_force_grad_a_##SFX(                                 \
      T* grad_net, const T* grad, const T* env_deriv, const int* nlist,        \
      int nloc, int nnei, int nframes) {                                       \
    deepmd::prod_force_grad_a_cpu(grad_net, grad, env_deriv, nlist, nloc,      \
                                  nnei, nframes);                              \
  }                                                                            \
  REF_EXPORT void ref_prod_virial_grad_a_##SFX(                                \
      T* grad_net, const T* grad, const T* env_deriv, const T* rij,            \
      const int* nlist, int nloc, int nnei) {                                  \
    deepmd::prod_virial_grad_a_cpu(grad_net, grad, env_deriv, rij, nlist,      \
                                   nloc, nnei);                                \
  }

REF_INSTANTIATE(double, f64)
REF_INSTANTIATE(float, f32)
