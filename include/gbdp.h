/*
 * gbdp.h - C ABI of the GB300 (sm_103a) se_e2_a descriptor library
 * (libgbdp.so).
 *
 * Plain pointers and sizes only.  Every device buffer (inputs, outputs and
 * workspace) is allocated by the caller; the library never calls cudaMalloc,
 * never synchronises the device and launches only on the stream it is given.
 * Return value: GBDP_OK (0), a positive GBDP_STATUS_* for a capacity problem
 * the caller can fix by retrying with more room, or a negative error code;
 * gbdp_last_error() then describes it.  No C++ exception crosses this ABI.
 *
 * Layouts follow the reference operator contract (DeePMD-kit, OutisLi fork):
 *   em          [nloc, nnei, 4]        (TF ProdEnvMatA "descrpt")
 *   em_deriv    [nloc, nnei, 4, 3]     ("descrpt_deriv")
 *   rij         [nloc, nnei, 3]
 *   nlist       [nloc, nnei] int32, -1 = empty slot, per-type sections
 *   table       [nspline, 6 * last_layer_size], coefficient-minor
 * with nnei = sum(sel).  Reference paths are relative to the reference
 * project root.
 */
#ifndef GBDP_H_
#define GBDP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gbdp_stream; /* == cudaStream_t */

#if defined(__GNUC__)
#define GBDP_API __attribute__((visibility("default")))
#else
#define GBDP_API
#endif

enum {
  GBDP_OK = 0,
  GBDP_STATUS_CAND_OVERFLOW = 1, /* a centre had more candidates than max_cand */
  GBDP_STATUS_EXT_OVERFLOW = 2,  /* more ghost atoms than the plan reserved  */
  GBDP_STATUS_TIMEOUT = 3,       /* a bounded device-side wait gave up       */
  GBDP_STATUS_BAD_INDEX = 4,     /* an input index was out of range          */
  GBDP_ERR_INVALID = -1,
  GBDP_ERR_CUDA = -2
};

/* Thread-local description of the last failure (empty string if none). */
GBDP_API const char* gbdp_last_error(void);
/* Library version, major * 10000 + minor * 100 + patch. */
GBDP_API int gbdp_version(void);

/* Self-test of the bounded device waits (no counterpart in the reference).
 * The tensor-core kernels wait on mbarriers for at most a fixed number of
 * polls; a wait that gives up raises GBDP_STATUS_TIMEOUT in the launch's
 * status word and the kernel returns instead of hanging.  This launches one
 * warp that completes a barrier phase with a 16-byte bulk copy of
 * result[0..3] (16-byte aligned device ints), then waits `limit` polls on
 * the next phase, which nothing completes.  Afterwards, in stream order:
 * result[0] = the copied result[0] + 1 (the satisfied wait saw the data),
 * result[1] = 0 (the second wait gave up), and *status (a device int the
 * caller zeroes) = GBDP_STATUS_TIMEOUT.  The GPU context stays usable. */
GBDP_API int gbdp_selftest_wait_timeout(int* status, int* result, long long limit,
                                        gbdp_stream stream);

/* ------------------------------------------------------------------------
 * Tabulated embedding + G^T.R contraction (compressed se_e2_a).
 * Replaces deepmd::tabulate_fusion_se_a_gpu / _grad_gpu / _grad_grad_gpu
 * (source/lib/include/tabulate.h:151-190; kernels
 * source/lib/src/gpu/tabulate.cu:196-503) as bound by the torch op
 * deepmd::tabulate_fusion_se_a (source/op/pt/tabulate_multi_device.cc:605-830,
 * :1498-1552).  table_info is a HOST array of 6 values
 * [lower, upper, max, stride0, stride1, check_freq], as the reference reads
 * it on the host (tabulate.cu:997-999).  em_x is [nloc, nnei], em
 * [nloc, nnei, 4], out / dy / dz_dy [nloc, 4, last_layer_size].
 * is_sorted != 0 enables the reference's trailing-padding fold.
 * ---------------------------------------------------------------------- */
GBDP_API int gbdp_tabulate_fusion_se_a_f32(float* out, const float* table, const float* table_info,
                                  const float* em_x, const float* em, int nloc, int nnei,
                                  int last_layer_size, int is_sorted, gbdp_stream stream);
GBDP_API int gbdp_tabulate_fusion_se_a_f64(double* out, const double* table, const double* table_info,
                                  const double* em_x, const double* em, int nloc, int nnei,
                                  int last_layer_size, int is_sorted, gbdp_stream stream);
GBDP_API int gbdp_tabulate_fusion_se_a_grad_f32(float* dy_dem_x, float* dy_dem, const float* table,
                                       const float* table_info, const float* em_x,
                                       const float* em, const float* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted, gbdp_stream stream);
GBDP_API int gbdp_tabulate_fusion_se_a_grad_f64(double* dy_dem_x, double* dy_dem, const double* table,
                                       const double* table_info, const double* em_x,
                                       const double* em, const double* dy, int nloc, int nnei,
                                       int last_layer_size, int is_sorted, gbdp_stream stream);
GBDP_API int gbdp_tabulate_fusion_se_a_grad_grad_f32(float* dz_dy, const float* table,
                                            const float* table_info, const float* em_x,
                                            const float* em, const float* dz_dy_dem_x,
                                            const float* dz_dy_dem, int nloc, int nnei,
                                            int last_layer_size, int is_sorted,
                                            gbdp_stream stream);
GBDP_API int gbdp_tabulate_fusion_se_a_grad_grad_f64(double* dz_dy, const double* table,
                                            const double* table_info, const double* em_x,
                                            const double* em, const double* dz_dy_dem_x,
                                            const double* dz_dy_dem, int nloc, int nnei,
                                            int last_layer_size, int is_sorted,
                                            gbdp_stream stream);

/* ------------------------------------------------------------------------
 * Neighbour plan for a packed batch of periodic frames.
 *
 * Frame f owns local atoms [atom_off, atom_off + nloc) of the packed
 * coordinate arrays and extended-atom slots [ext_off, ext_off + ext_cap).
 * Within a frame, extended atoms are numbered exactly as the reference's
 * copy_coord orders them (source/lib/src/neighbor_list.cc:745-845): local
 * atoms first, then the ghost images cell by cell.  The cell geometry is the
 * reference's (ncell = floor(face distance / rcut), ngcell = int(rcut / cell)
 * + 1).  gbdp_nbr_plan_make fills the plan and the frame table on the host;
 * the caller copies the frame table (plan->nframes structs, plain bytes) to
 * device memory and passes that copy to the device entry points.  For float
 * coordinates pass the float box values (exactly widened to double): the
 * reference builds the cell grid and ghost shifts from the float box
 * (source/lib/src/coord.cc:42-47).
 * ---------------------------------------------------------------------- */
typedef struct gbdp_nbr_frame {
  double box[9];   /* rows are the cell vectors                          */
  double rec[9];   /* reciprocal (fractional = rec * phys), double       */
  float boxf[9];   /* the same in float, for float coordinates           */
  float recf[9];
  int ncell[3];    /* local cells per dimension                          */
  int ngcell[3];   /* ghost cell layers per dimension                    */
  int stencil[3];  /* neighbour-cell half width per dimension            */
  int nloc;        /* local atoms                                        */
  int atom_off;    /* first local atom in the packed arrays              */
  int cell_off;    /* first local cell                                   */
  int ext_cell_off;/* first extended cell                                */
  int ext_off;     /* first extended-atom slot                           */
  int ext_cap;     /* extended-atom slots reserved (upper bound of nall) */
  int subcell;     /* bit d: the neighbour search scans half cells along d */
} gbdp_nbr_frame;

typedef struct gbdp_nbr_plan {
  int nframes;
  int nloc_total;
  int ncell_total;     /* local cells, all frames    */
  int next_cell_total; /* extended cells, all frames */
  int ext_total;       /* extended-atom slots        */
  int max_cand;        /* candidates per centre kept on chip */
  float rcut;
  int pad0;
} gbdp_nbr_plan;

/* Fill plan and frames[nframes] from per-frame atom counts and HOST boxes
 * (nframes x 9, row vectors).  max_cand <= 0 selects the default (512). */
GBDP_API int gbdp_nbr_plan_make(gbdp_nbr_plan* plan, gbdp_nbr_frame* frames, int nframes,
                       const int* nloc, const double* boxes, float rcut, int max_cand);

/* Device workspace bytes for gbdp_prod_env_mat_a_* with this plan. */
GBDP_API size_t gbdp_env_workspace_bytes(const gbdp_nbr_plan* plan, int fp64);

/* ------------------------------------------------------------------------
 * Environment matrix with the internal periodic neighbour build.
 * Replaces deepmd::prod_env_mat_a_gpu (source/lib/include/prod_env_mat.h:47-65)
 * together with the TF ProdEnvMatA op's internal-PBC mode
 * (source/op/tf/prod_env_mat_multi_device.cc:11-28, :417-438 nei_mode 1:
 * normalize_coord, copy_coord, build_nlist, format_nlist, env mat, map).
 *
 * Inputs (device, packed over frames): coord [nloc_total, 3], atype
 * [nloc_total] (type < 0 atoms are never neighbours), avg / std
 * [ntypes, nnei * 4].  sel is a HOST array of ntypes section sizes.
 * Outputs (device): em, nlist (frame-local indices of LOCAL atoms, the TF
 * op's mapped form), and optionally (NULL to skip) em_deriv, rij and
 * nlist_ext (frame-local extended indices).  ext_coord [ext_total, 3],
 * ext_type, ext_map [ext_total] receive the extended system (slots past a
 * frame's nall are left untouched); ext_nall [nframes] its atom count.
 * Neighbour order within a type section is (float r^2, extended index)
 * ascending, bit-exact against format_nlist_cpu (source/lib/src/fmt_nlist.cc:
 * 98-143).  A GBDP_STATUS_* code is also written to the first int of the
 * workspace; read it with gbdp_env_status after the stream has run.
 * ---------------------------------------------------------------------- */
GBDP_API int gbdp_prod_env_mat_a_f32(float* em, float* em_deriv, float* rij, int* nlist, int* nlist_ext,
                            float* ext_coord, int* ext_type, int* ext_map, int* ext_nall,
                            const float* coord, const int* atype, const float* avg,
                            const float* std, const gbdp_nbr_plan* plan,
                            const gbdp_nbr_frame* frames_dev, float rcut_smth, const int* sel,
                            int ntypes, void* workspace, size_t workspace_bytes,
                            gbdp_stream stream);
GBDP_API int gbdp_prod_env_mat_a_f64(double* em, double* em_deriv, double* rij, int* nlist,
                            int* nlist_ext, double* ext_coord, int* ext_type, int* ext_map,
                            int* ext_nall, const double* coord, const int* atype,
                            const double* avg, const double* std, const gbdp_nbr_plan* plan,
                            const gbdp_nbr_frame* frames_dev, float rcut_smth, const int* sel,
                            int ntypes, void* workspace, size_t workspace_bytes,
                            gbdp_stream stream);

/* prod_env_mat_a from an external neighbour list: the forward_lower path of
 * the PyTorch model (an MD engine hands over extended coordinates and an
 * unsorted rcut + skin list).  Replaces the descriptor's own formatting and
 * env matrix there: deepmd/pt/model/model/make_model.py:541-598 (_format_nlist
 * with the forced sort a compressed se_e2_a asks for,
 * need_sorted_nlist_for_lower in deepmd/pt/model/descriptor/se_a.py:872-883),
 * deepmd/pt/utils/nlist.py:304-337 (nlist_distinguish_types), then the env
 * rows of env_mat_a_cpu (source/lib/src/env_mat.cc:122-226) normalised as
 * prod_env_mat.cc:84-100.  Per frame f and local atom i (the first nloc
 * extended atoms): the listed j >= 0 at rr = |x_i - x_j| (coordinate type),
 * rr > rcut dropped, ascending rr (ties by list position), the nearest
 * sum(sel) kept, then the first sel[t] of type t fill section t.
 * Device inputs: ext_coord [nframes, nall, 3], ext_type [nframes, nall],
 * nlist_in [nframes, nloc, nnei_in] (extended indices, -1 padding,
 * nnei_in <= 4096), avg/std [ntypes, sum(sel) * 4]; sel on the host.
 * Outputs: em [nframes * nloc, sum(sel) * 4], em_deriv (x3, may be NULL),
 * rij (x3/4, may be NULL), nlist [nframes * nloc, sum(sel)] in the extended
 * index space; status (device int, may be NULL) becomes
 * GBDP_STATUS_BAD_INDEX if a listed index is >= nall. */
GBDP_API int gbdp_prod_env_mat_a_nlist_f32(float* em, float* em_deriv, float* rij, int* nlist,
                                           int* status, const float* ext_coord,
                                           const int* ext_type, const int* nlist_in,
                                           const float* avg, const float* std, int nframes,
                                           int nloc, int nall, int nnei_in, float rcut,
                                           float rcut_smth, const int* sel, int ntypes,
                                           gbdp_stream stream);
GBDP_API int gbdp_prod_env_mat_a_nlist_f64(double* em, double* em_deriv, double* rij,
                                           int* nlist, int* status, const double* ext_coord,
                                           const int* ext_type, const int* nlist_in,
                                           const double* avg, const double* std, int nframes,
                                           int nloc, int nall, int nnei_in, float rcut,
                                           float rcut_smth, const int* sel, int ntypes,
                                           gbdp_stream stream);

/* Verlet-list (skin) form of gbdp_prod_env_mat_a_*, for MD steps that
 * rebuild the neighbour list every few steps, as the reference's LAMMPS
 * path reuses an rcut + skin list between rebuilds
 * (source/api_cc/src/DeepPotPT.cc:311-330, list formatted by
 * deepmd/pt/model/model/make_model.py:541-598 and sorted as se_a asks,
 * deepmd/pt/model/descriptor/se_a.py:872-883).  No single reference
 * function: it combines the periodic build with the formatting of a stored
 * list.  The plan is made with the cutoff rcut + skin (its cells and ghost
 * images cover that range); `rcut` is the model cutoff (<= plan->rcut).
 *   rebuild != 0  the ghost images and cells are built as by
 *                 gbdp_prod_env_mat_a_*, ext_src / ext_shift record each
 *                 filled extended slot's local source atom (packed index)
 *                 and its offset from that atom's coordinate, and vlist
 *                 [nloc_total, vcap] / vcnt [nloc_total] receive every
 *                 extended atom within plan->rcut of each centre;
 *   rebuild == 0  ext_coord is refreshed as coord[ext_src] + ext_shift and
 *                 nothing else is rebuilt.
 * Either way the outputs are formed from the stored candidates within
 * rcut of the current coordinates, in the canonical order (type, float
 * r^2, extended index; indices of the last rebuild).  A centre with more
 * than vcap candidates raises GBDP_STATUS_CAND_OVERFLOW (rebuild again with
 * a larger vcap).  The caller keeps vlist, vcnt, ext_shift [ext_total, 3],
 * ext_src [ext_total], the outputs and the workspace between calls and
 * rebuilds before the atoms have moved by more than half the skin. */
GBDP_API int gbdp_prod_env_mat_a_skin_f32(
    float* em, float* em_deriv, float* rij, int* nlist, int* nlist_ext, float* ext_coord,
    int* ext_type, int* ext_map, int* ext_nall, const float* coord, const int* atype,
    const float* avg, const float* std, const gbdp_nbr_plan* plan,
    const gbdp_nbr_frame* frames_dev, float rcut, float rcut_smth, const int* sel, int ntypes,
    int rebuild, int* vlist, int* vcnt, int vcap, float* ext_shift, int* ext_src,
    void* workspace, size_t workspace_bytes, gbdp_stream stream);
GBDP_API int gbdp_prod_env_mat_a_skin_f64(
    double* em, double* em_deriv, double* rij, int* nlist, int* nlist_ext, double* ext_coord,
    int* ext_type, int* ext_map, int* ext_nall, const double* coord, const int* atype,
    const double* avg, const double* std, const gbdp_nbr_plan* plan,
    const gbdp_nbr_frame* frames_dev, float rcut, float rcut_smth, const int* sel, int ntypes,
    int rebuild, int* vlist, int* vcnt, int vcap, double* ext_shift, int* ext_src,
    void* workspace, size_t workspace_bytes, gbdp_stream stream);

/* Allocation-free variant of gbdp_prod_env_mat_a_f32 (float only).  It has
 * no counterpart in the reference.  It is for callers that cannot allocate
 * device memory at the point of the call: a host MD engine that owns all
 * device memory through its own pool and forbids driver allocations inside
 * its force callback, or code that runs while a stream is being captured,
 * where cudaMalloc is not allowed.  Instead of a caller workspace it uses a
 * built-in 16 MiB device scratch array that every GPU loading the library
 * holds until exit (enough for a batch of roughly 100k atoms at water
 * density); a batch whose workspace would exceed 16 MiB - 64 KiB, or with
 * more than 234 frames (the 64 KiB frame table holds 234 records of 280
 * bytes), is rejected with GBDP_ERR_INVALID and a message before any device
 * work, as is every argument gbdp_prod_env_mat_a_f32 would reject.
 * The frame table is passed on the HOST (frames_host) and copied into the
 * scratch in stream order; `status` is a caller-provided device int that
 * receives the device status word (GBDP_OK or a GBDP_STATUS_* code) in
 * stream order.  Other arguments and outputs are those of
 * gbdp_prod_env_mat_a_f32.
 * Every call made outside stream capture looks up the scratch array's
 * device address for the current device (cudaGetSymbolAddress); a call
 * under capture reuses the address of the last uncaptured call on that
 * device, so make one call on each device before capturing.  A captured
 * call re-reads frames_host on every replay: it must then be pinned host
 * memory that outlives the graph.  All calls share the one array and it
 * keeps the last call's contents (counters are cleared at the start of
 * every call): calls that overlap on the GPU, on any stream, race with each
 * other.  The function itself never calls cudaMalloc or cudaFree. */
GBDP_API int gbdp_prod_env_mat_a_noalloc_f32(
    float* em, float* em_deriv, float* rij, int* nlist, int* nlist_ext, float* ext_coord,
    int* ext_type, int* ext_map, int* ext_nall, int* status, const float* coord,
    const int* atype, const float* avg, const float* std, const gbdp_nbr_plan* plan,
    const gbdp_nbr_frame* frames_host, float rcut_smth, const int* sel, int ntypes,
    gbdp_stream stream);

/* Synchronise `stream` and return the device status word of an env-mat
 * workspace (GBDP_OK or a GBDP_STATUS_* code). */
GBDP_API int gbdp_env_status(const void* workspace, gbdp_stream stream);

/* ------------------------------------------------------------------------
 * Force and virial from the derivative of the energy wrt the env matrix.
 * Replace deepmd::prod_force_a_gpu (source/lib/include/prod_force.h:72-80,
 * kernels source/lib/src/gpu/prod_force.cu:4-131) and
 * deepmd::prod_virial_a_gpu (source/lib/include/prod_virial.h:30-38,
 * source/lib/src/gpu/prod_virial.cu:4-135), bound by the TF ops ProdForceSeA
 * (source/op/tf/prod_force_multi_device.cc:6-14) and ProdVirialSeA
 * (source/op/tf/prod_virial_multi_device.cc:5-15).
 * net_deriv [nframes, nloc, nnei*4], env_deriv [nframes, nloc, nnei*4, 3],
 * rij [nframes, nloc, nnei, 3], nlist [nframes, nloc, nnei] (indices in
 * [0, nall)), force [nframes, nall, 3], virial [nframes, 9], atom_virial
 * [nframes, nall, 9].  deterministic != 0 gathers through a reverse
 * neighbour list (bitwise reproducible); 0 scatters with atomics (FP32
 * forces accumulate in 16-byte padded rows of the workspace, one vector
 * reduction a pair, then are compacted into `force`; the workspace size
 * below includes those rows).
 * ---------------------------------------------------------------------- */
GBDP_API size_t gbdp_prod_workspace_bytes(int nframes, int nloc, int nall, int nnei, int deterministic);
GBDP_API int gbdp_prod_force_a_f32(float* force, const float* net_deriv, const float* env_deriv,
                          const int* nlist, int nloc, int nall, int nnei, int nframes,
                          int deterministic, void* workspace, size_t workspace_bytes,
                          gbdp_stream stream);
GBDP_API int gbdp_prod_force_a_f64(double* force, const double* net_deriv, const double* env_deriv,
                          const int* nlist, int nloc, int nall, int nnei, int nframes,
                          int deterministic, void* workspace, size_t workspace_bytes,
                          gbdp_stream stream);
GBDP_API int gbdp_prod_virial_a_f32(float* virial, float* atom_virial, const float* net_deriv,
                           const float* env_deriv, const float* rij, const int* nlist,
                           int nloc, int nall, int nnei, int nframes, int deterministic,
                           void* workspace, size_t workspace_bytes, gbdp_stream stream);
GBDP_API int gbdp_prod_virial_a_f64(double* virial, double* atom_virial, const double* net_deriv,
                           const double* env_deriv, const double* rij, const int* nlist,
                           int nloc, int nall, int nnei, int nframes, int deterministic,
                           void* workspace, size_t workspace_bytes, gbdp_stream stream);

/* Force and virial in one pass over net_deriv / env_deriv / nlist (no
 * counterpart in the reference, which runs ProdForceSeA and ProdVirialSeA
 * as two ops reading the same inputs): the outputs of gbdp_prod_force_a_*
 * and gbdp_prod_virial_a_* with the same arguments, the 80 B a slot of
 * net_deriv, env_deriv, nlist (and 12 B of rij) read once instead of twice.
 * Same workspace (gbdp_prod_workspace_bytes), modes and alignment rules. */
GBDP_API int gbdp_prod_force_virial_a_f32(float* force, float* virial, float* atom_virial,
                                          const float* net_deriv, const float* env_deriv,
                                          const float* rij, const int* nlist, int nloc, int nall,
                                          int nnei, int nframes, int deterministic,
                                          void* workspace, size_t workspace_bytes,
                                          gbdp_stream stream);
GBDP_API int gbdp_prod_force_virial_a_f64(double* force, double* virial, double* atom_virial,
                                          const double* net_deriv, const double* env_deriv,
                                          const double* rij, const int* nlist, int nloc, int nall,
                                          int nnei, int nframes, int deterministic,
                                          void* workspace, size_t workspace_bytes,
                                          gbdp_stream stream);

/* Backward of the two ops wrt net_deriv (second order of the env-mat
 * derivative).  Replace deepmd::prod_force_grad_a_gpu
 * (source/lib/include/prod_force_grad.h, source/lib/src/gpu/
 * prod_force_grad.cu:10-145) and deepmd::prod_virial_grad_a_gpu
 * (source/lib/include/prod_virial_grad.h, source/lib/src/gpu/
 * prod_virial_grad.cu:14-130).  grad [nframes, nloc, 3] (force) or
 * [nframes, 9] (virial); grad_net [nframes, nloc, nnei*4].  For the force
 * version, neighbour indices >= nloc are folded with j % nloc as the
 * reference does (prod_force_grad.cc:54-57). */
GBDP_API int gbdp_prod_force_grad_a_f32(float* grad_net, const float* grad, const float* env_deriv,
                               const int* nlist, int nloc, int nnei, int nframes,
                               gbdp_stream stream);
GBDP_API int gbdp_prod_force_grad_a_f64(double* grad_net, const double* grad, const double* env_deriv,
                               const int* nlist, int nloc, int nnei, int nframes,
                               gbdp_stream stream);
GBDP_API int gbdp_prod_virial_grad_a_f32(float* grad_net, const float* grad, const float* env_deriv,
                                const float* rij, const int* nlist, int nloc, int nnei,
                                int nframes, gbdp_stream stream);
GBDP_API int gbdp_prod_virial_grad_a_f64(double* grad_net, const double* grad, const double* env_deriv,
                                const double* rij, const int* nlist, int nloc, int nnei,
                                int nframes, gbdp_stream stream);


/* ------------------------------------------------------------------------
 * Fused compressed se_e2_a descriptor (the batched "chosen form").
 * Forward: X [nloc, 4, M] = sum over sections of the tabulated embedding
 * contracted with the env rows, / nnei; D [nloc, M * axis_neuron] =
 * X^T X[:, :axis_neuron] (DescrptBlockSeA.forward with compression,
 * deepmd/pt/model/descriptor/se_a.py:786-866, tables as bound through
 * deepmd::tabulate_fusion_se_a).  tables: HOST array of device table
 * pointers, one per embedding net (ntypes nets if type_one_side, else
 * ntypes^2 indexed tj * ntypes + ti), each in the k-planar layout written
 * by gbdp_table_to_planar_* and 128-byte aligned; table_infos: HOST
 * [n_tables * 6];
 * sel: HOST [ntypes].  em comes from gbdp_prod_env_mat_a_*.  d_row (device,
 * may be NULL for the identity) gives the row of D / dE_dD that belongs to
 * atom i, so that a caller can keep each type's rows contiguous; it must
 * hold a valid row for every atom, an atom of type < 0 included (the
 * forward writes its row, from zero sums).
 * Backward: from dE/dD, force [nloc, 3] (zeroed here, local indices, packed
 * frames) and virial_acc [nframes, 9] (double, zeroed here) get the
 * contributions of every real neighbour, the env-matrix derivative being
 * recomputed from ext_coord (prod_force.cc:22-72, prod_virial.cc:22-68
 * semantics); inv_std [ntypes, nnei * 4] is 1 / dstd.  force_fx (device,
 * may be NULL): with it, every force and virial contribution is summed in
 * 64-bit fixed point (forces on a grid of 2^-32 eV/A in FP32, 2^-40 in FP64;
 * virials 2^-32 / 2^-36 eV) in force_fx [nloc, 3] and in virial_acc, then
 * written as values, so that the results are the same bits on every run;
 * without it the sums are floating-point atomics.  atom_frame [nloc], frame_atom_off / frame_ext_off [nframes]
 * are device arrays describing the packed batch (see gbdp_nbr_frame).
 * ---------------------------------------------------------------------- */
/* The fused descriptor kernels read the tables of tabulate_fusion_se_a
 * ([nspline, 6 M], coefficient-minor, as above) in a k-planar copy: row r
 * holds 3 planes of pitch P elements (P = 2 M rounded up to 128 bytes),
 * plane p the pairs (a_2p, a_2p+1) of output k at 2 k, so that consecutive
 * k are adjacent in memory.  No reference counterpart: a layout choice of
 * this library.  row_elems = 3 P for the element size (4 or 8 bytes); dst
 * holds nrow * row_elems elements, 128-byte aligned; src and dst device. */
GBDP_API size_t gbdp_table_planar_row_elems(int last_layer_size, int elem_bytes);
GBDP_API int gbdp_table_to_planar_f32(float* dst, const float* src, int nrow,
                                      int last_layer_size, gbdp_stream stream);
GBDP_API int gbdp_table_to_planar_f64(double* dst, const double* src, int nrow,
                                      int last_layer_size, gbdp_stream stream);

GBDP_API int gbdp_se_a_descriptor_fwd_f32(float* X, float* D, const float* em, const int* atype,
                                          const int* d_row, const float* const* tables, const float* table_infos,
                                          int ntypes, const int* sel, int type_one_side,
                                          int nloc, int last_layer_size, int axis_neuron,
                                          gbdp_stream stream);
GBDP_API int gbdp_se_a_descriptor_fwd_f64(double* X, double* D, const double* em,
                                          const int* atype, const int* d_row,
                                          const double* const* tables,
                                          const double* table_infos, int ntypes, const int* sel,
                                          int type_one_side, int nloc, int last_layer_size,
                                          int axis_neuron, gbdp_stream stream);
GBDP_API int gbdp_se_a_descriptor_bwd_f32(
    float* force, double* virial_acc, const float* X, const float* dE_dD, const int* d_row,
    const float* em,
    const int* nlist_ext, const float* ext_coord, const int* ext_map, const int* atype,
    const float* inv_std, const int* atom_frame, const int* frame_atom_off, const int* frame_ext_off,
    const float* const* tables, const float* table_infos, int ntypes, const int* sel,
    int type_one_side, float rcut_smth, float rcut, int nloc, int nframes, int last_layer_size,
    int axis_neuron, long long* force_fx, gbdp_stream stream);
GBDP_API int gbdp_se_a_descriptor_bwd_f64(
    double* force, double* virial_acc, const double* X, const double* dE_dD, const int* d_row,
    const double* em,
    const int* nlist_ext, const double* ext_coord, const int* ext_map, const int* atype,
    const double* inv_std, const int* atom_frame, const int* frame_atom_off,
    const int* frame_ext_off, const double* const* tables, const double* table_infos,
    int ntypes, const int* sel, int type_one_side, float rcut_smth, float rcut, int nloc,
    int nframes, int last_layer_size, int axis_neuron, long long* force_fx, gbdp_stream stream);

/* Frame energies of a packed batch: E [nframes] (FP64, zeroed here) = the
 * sum of the per-row energies ae [nrows] whose frame_of_row [nrows] is the
 * frame (rows with -1 are skipped).  Device pointers.  The energy reduction
 * of the reference's model output (atomic energies summed per frame in the
 * FP64 energy precision, deepmd/pt/model/model/transform_output.py:165,181).
 * deterministic != 0: the partial sums are added in 64-bit fixed point
 * (grid 2^-30 eV), so that E is the same bits on every run. */
GBDP_API int gbdp_frame_energy_f32(double* E, const float* ae, const int* frame_of_row, int nrows,
                                   int nframes, int deterministic, gbdp_stream stream);
GBDP_API int gbdp_frame_energy_f64(double* E, const double* ae, const int* frame_of_row,
                                   int nrows, int nframes, int deterministic, gbdp_stream stream);

/* ------------------------------------------------------------------------
 * Fitting net of one atom type: per-atom energy e = H_L w_out + b_out and
 * dE/dD for every row of D [n, widths[0]] (deepmd/pt/model/task/
 * fitting.py:734-899; hidden layer l: H_l = tanh(H_{l-1} W_l + b_l) * idt_l,
 * plus H_{l-1} when widths[l] == widths[l-1]).  w, b, idt are HOST arrays of
 * n_hidden device pointers (W_l row-major [widths[l-1], widths[l]]; an idt
 * entry, or idt itself, may be NULL); w_out [widths[n_hidden]] device.
 * gemm_mode selects the cuBLAS compute type of the six GEMMs: 0 FP32
 * (pedantic), 1 FP32 emulated with BF16x9 on tensor cores, 2 TF32, 3 BF16.
 * The first call on a device creates its cuBLAS handle: make it before any
 * stream capture. */
GBDP_API size_t gbdp_fitting_workspace_bytes(int n, const int* widths, int n_hidden,
                                             const float* const* idt);
GBDP_API int gbdp_fitting_fwd_bwd_f32(float* e, float* dD, const float* D, int n,
                                      const int* widths, int n_hidden, const float* const* w,
                                      const float* const* b, const float* const* idt,
                                      const float* w_out, float b_out, int gemm_mode,
                                      void* workspace, size_t workspace_bytes,
                                      gbdp_stream stream);

/* As gbdp_se_a_descriptor_fwd_f32, but D is written split for the tensor-
 * core fitting, as two FP16 arrays (IEEE binary16, [nrows, M * axis_neuron]
 * each) under a power-of-two scale per row: with c = 2^s the scale of row r,
 * D_hi = fp16(c D) and D_lo = fp16(c D - D_hi) (round to nearest), and
 * D_rscale[r] = 1 / c.  c is chosen from the Cauchy-Schwarz bound
 * |D_ka| <= |X_k| |X_a| so that c |D| < 2^15.  Rows no atom maps to are not
 * written. */
GBDP_API int gbdp_se_a_descriptor_fwd_split_f32(
    float* X, void* D_hi, void* D_lo, float* D_rscale, const float* em, const int* atype, const int* d_row,
    const float* const* tables, const float* table_infos, int ntypes, const int* sel,
    int type_one_side, int nloc, int last_layer_size, int axis_neuron, gbdp_stream stream);

/* ------------------------------------------------------------------------
 * Fitting nets on the tensor cores (tcgen05 kind::f16, each FP32 operand as
 * a scaled FP16 hi/lo pair, which keeps FP32-level accuracy), for the
 * se_e2_a fitting shape 1600 -> 240 -> 240 -> 240 -> 1 (layers 2 and 3
 * with time step and skip).
 * Rows are grouped by atom type: type t owns rows [row_off[t],
 * row_off[t] + nrows[t]) of every activation, row_off[t] a multiple of 128,
 * row_off[ntypes] the padded total (also a multiple of 128).  D is given
 * split with its per-row inverse scales, as
 * gbdp_se_a_descriptor_fwd_split_f32 writes it.  Per type (device
 * pointers; FP16 images 16-byte aligned, FP32 arrays 16-byte aligned):
 *   w_hi/w_lo[l]   W_l [in, out] with row i scaled by 2^u_i, split
 *   wt_hi/wt_lo[l] W_l^T [out, in] with row j scaled by 2^v_j, split
 *   cs_fwd[l]      [out]: 2^-(v_j + s_in(l)), s_in = 0, s_H1, s_H2
 *   cs_bwd[l]      [in]:  2^-(u_i + s_g(l)),  s_g = s_GZ1, s_GZ2, s_GZ3
 *   act_scale      2^s of the split activations H1, H2, GZ3, GZ2, GZ1 in
 *                  that order, each bringing a bound on the activation's
 *                  magnitude below 2^15 (dpmd_public_gb300.se_a builds all
 *                  of these from the parameters)
 *   b[l]; idt[l] (NULL for layer 0); w_out [240]; b_out on the host.
 * Outputs: e [rows] per-row energy (0 on padding rows), dE_dD [rows, 1600].
 * ---------------------------------------------------------------------- */
typedef struct gbdp_fit_tc_net {
  const void* w_hi[3];
  const void* w_lo[3];
  const void* wt_hi[3];
  const void* wt_lo[3];
  const float* cs_fwd[3];
  const float* cs_bwd[3];
  float act_scale[5];
  const float* b[3];
  const float* idt[3];
  const float* w_out;
  float b_out;
} gbdp_fit_tc_net;

GBDP_API size_t gbdp_fitting_tc_workspace_bytes(int rows);
GBDP_API int gbdp_fitting_tc_f32(float* e, float* dE_dD, const void* D_hi, const void* D_lo,
                                 const float* D_rscale, int ntypes, const int* nrows,
                                 const int* row_off, const gbdp_fit_tc_net* nets,
                                 void* workspace, size_t workspace_bytes, gbdp_stream stream);
/* Synchronise `stream`; device status word of the last gbdp_fitting_tc_f32
 * run on this workspace (GBDP_OK or GBDP_STATUS_TIMEOUT). */
GBDP_API int gbdp_fitting_tc_status(const void* workspace, int rows, gbdp_stream stream);

/* Launch-shape control of the tensor-core fitting (no counterpart in the
 * reference): the four K-240 layers (F2, F3, B3, B2) run as one CTA per
 * 128 x 80 tile, two per SM, while a layer has fewer than `tiles_per_sm`
 * tiles per SM (default 32), and on the persistent kernel (one CTA per SM,
 * double-buffered accumulators) from there on.  Process-wide. */
GBDP_API void gbdp_fitting_tc_set_persistent_min_tiles(int tiles_per_sm);

/* ---- launch-shape autotuning ----------------------------------------------
 * The fused descriptor kernels (the gbdp_se_a_descriptor_ fwd and bwd entry
 * points) run 1, 2 or 4 centre atoms per CTA, and the FP32 backward 1 or 2
 * neighbours in flight per 16-lane group.  With autotuning on, the first
 * call for a shape key
 * (kernel, dtype, last_layer_size, nnei, floor(log2 nloc)) that is not under
 * stream capture times every choice on the caller's stream (it synchronises
 * that stream) and keeps the fastest in a mutex-guarded cache; later calls
 * with that key, captured or not, use it.  Off by default (4 per CTA, 1
 * neighbour in flight).
 * No reference counterpart.  gbdp_autotune_report writes one line per tuned
 * key into buf (NUL-terminated, at most len bytes) and returns the full
 * length. */
GBDP_API void gbdp_set_autotune(int on);
GBDP_API int gbdp_autotune_report(char* buf, int len);

/* ---- uncompressed embedding net on the tensor cores (BF16) ----------------
 * Replaces the plain-form embedding of DescrptBlockSeA.forward
 * (deepmd/pt/model/descriptor/se_a.py:750-866; EmbeddingNet / MLPLayer,
 * deepmd/pt/model/network/mlp.py:188-219) together with its G^T R
 * contraction and D = X^T X[:, :axis]: layers 2 and 3 as BF16 tcgen05 MMAs
 * with FP32 accumulation, everything else in FP32.  Built for embedding
 * widths 25-50-100 and 3-6-12 (tanh, identity / [x, x] skips).
 *
 * nets: one block of gbdp_embed_tc_net_bytes() per net (net index tj when
 * type_one_side, else tj * ntypes + ti), 16-byte aligned, holding the bf16
 * weight images and FP32 parameters in the layout the kernels stage (built
 * once per model on the host).  units: [nunits, 2] pairs of atoms of one
 * centre type (second entry -1 when absent), covering every local atom once.
 * sel: host array of ntypes.  status: device int, GBDP_STATUS_TIMEOUT if a
 * tensor-core wait gave up.
 *
 * forward:  X [nloc, 4, n3] (sums / nnei), D [rows, n3 * axis] at row drow[i]
 *           (drow null: row i), FP32; or, with D_lo and D_rscale given, D
 *           split for the tensor-core fitting (D and D_lo FP16 hi / lo
 *           parts, D_rscale per-row inverse scales, as
 *           gbdp_se_a_descriptor_fwd_split_f32 writes them).
 * backward: from dE/dD (same rows), the gradient wrt the env matrix
 *           net_deriv [nloc, nnei, 4] (every slot written); dx_work is
 *           caller scratch of nloc * 4 * n3 floats. */
GBDP_API size_t gbdp_embed_tc_net_bytes(void);
GBDP_API int gbdp_embed_fwd_tc_bf16(float* X, void* D, void* D_lo, float* D_rscale,
                                    const int* drow, const float* em, const int* atype,
                                    const int* units, int nunits, const void* nets, int ntypes,
                                    const int* sel,
                                    int type_one_side, int nloc, int nnei, int n1, int n2, int n3,
                                    int axis, int* status, gbdp_stream stream);
GBDP_API int gbdp_embed_bwd_tc_bf16(float* net_deriv, float* dx_work, const float* dD,
                                    const float* X, const int* drow, const float* em,
                                    const int* atype, const int* units, int nunits,
                                    const void* nets, int ntypes, const int* sel,
                                    int type_one_side, int nloc, int nnei, int n1, int n2, int n3,
                                    int axis, int* status, gbdp_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* GBDP_H_ */
