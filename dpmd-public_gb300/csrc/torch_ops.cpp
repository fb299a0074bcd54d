// libtorch registration of the deepmd operators on this path, for C++
// processes that run TorchScript models (DeepPotPT::compute,
// source/api_cc/src/DeepPotPT.cc:171-410, as LAMMPS does).  It stands in for
// the reference's libdeepmd_op_pt.so on the se_e2_a path: it owns
// TORCH_LIBRARY(deepmd) with enable_mpi (source/op/pt/print_summary.cc:14;
// deepmd/pt/cxx_op.py:22-60 skips loading the reference's library when it is
// present) and tabulate_fusion_se_a with the reference's schema and
// autograd (source/op/pt/tabulate_multi_device.cc:605-830,1498-1552):
// forward -> descriptor [nloc, 4, M]; backward -> grads for em_x and em;
// the grad op's backward -> the grad for dy only.  Every call goes to
// libgbdp.so on the current CUDA stream; CPU tensors raise.
#include <c10/cuda/CUDAStream.h>
#include <torch/autograd.h>
#include <torch/library.h>
#include <torch/types.h>

#include <string>
#include <vector>

#include "gbdp.h"

namespace {

using torch::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

void check_rc(int rc, const char* what) {
  TORCH_CHECK(rc == GBDP_OK, what, " failed (", rc, "): ", gbdp_last_error());
}

void need_cuda(const Tensor& t) {
  TORCH_CHECK(t.is_cuda(),
              "the GB300 deepmd operators run on CUDA tensors only (got a CPU tensor); "
              "there is no CPU fallback");
}

gbdp_stream cur_stream(const Tensor& t) {
  return reinterpret_cast<gbdp_stream>(c10::cuda::getCurrentCUDAStream(t.device().index()).stream());
}

// table_info is read on the host, as the reference's kernels do (tabulate.cu
// reads it through a host pointer); check the table covers every row it
// addresses
template <typename T>
std::vector<T> host_info(const Tensor& info, const Tensor& table) {
  Tensor h = info.detach().to(torch::kCPU, torch::kFloat64).contiguous();
  TORCH_CHECK(h.numel() >= 5, "table_info must hold at least 5 values");
  const double* v = h.data_ptr<double>();
  TORCH_CHECK(v[3] > 0 && v[4] > 0, "table strides must be positive");
  std::vector<T> out(v, v + h.numel());
  const T lo = (T)v[0], up = (T)v[1], mx = (T)v[2], s0 = (T)v[3], s1 = (T)v[4];
  const long last = (long)((T)(up - lo) / s0) + (long)((T)(mx - up) / s1) - 1;
  TORCH_CHECK(table.size(0) > last, "table has ", table.size(0),
              " rows but table_info addresses row ", last);
  return out;
}

Tensor tab_forward(const Tensor& table_in, const Tensor& info, const Tensor& em_x_in,
                   const Tensor& em_in, int64_t M) {
  need_cuda(table_in);
  need_cuda(em_x_in);
  need_cuda(em_in);
  TORCH_CHECK(table_in.dim() == 2, "Dim of table should be 2");
  TORCH_CHECK(em_x_in.dim() == 2, "Dim of input should be 2");
  TORCH_CHECK(em_in.dim() == 3, "Dim of input should be 3");
  const Tensor table = table_in.contiguous();
  const Tensor em_x = em_x_in.to(table.scalar_type()).contiguous();
  const Tensor em = em_in.to(table.scalar_type()).contiguous();
  const int nloc = (int)em.size(0), nnei = (int)em.size(1);
  Tensor out = torch::empty({nloc, 4, M}, table.options());
  int rc;
  if (table.scalar_type() == torch::kFloat64) {
    auto hi = host_info<double>(info, table);
    rc = gbdp_tabulate_fusion_se_a_f64(out.data_ptr<double>(), table.data_ptr<double>(), hi.data(),
                                       em_x.data_ptr<double>(), em.data_ptr<double>(), nloc, nnei,
                                       (int)M, 1, cur_stream(table));
  } else {
    TORCH_CHECK(table.scalar_type() == torch::kFloat32, "table must be float32 or float64");
    auto hi = host_info<float>(info, table);
    rc = gbdp_tabulate_fusion_se_a_f32(out.data_ptr<float>(), table.data_ptr<float>(), hi.data(),
                                       em_x.data_ptr<float>(), em.data_ptr<float>(), nloc, nnei,
                                       (int)M, 1, cur_stream(table));
  }
  check_rc(rc, "tabulate_fusion_se_a");
  return out;
}

std::vector<Tensor> tab_grad(const Tensor& table_in, const Tensor& info, const Tensor& em_x_in,
                             const Tensor& em_in, const Tensor& dy_in) {
  need_cuda(dy_in);
  TORCH_CHECK(dy_in.dim() == 3, "Dim of dy_tensor should be 3");
  const Tensor table = table_in.contiguous();
  const auto st = table.scalar_type();
  const Tensor em_x = em_x_in.to(st).contiguous();
  const Tensor em = em_in.to(st).contiguous();
  const Tensor dy = dy_in.to(st).contiguous();
  const int nloc = (int)em.size(0), nnei = (int)em.size(1), M = (int)dy.size(2);
  Tensor gx = torch::empty_like(em_x), gm = torch::empty_like(em);
  int rc;
  if (st == torch::kFloat64) {
    auto hi = host_info<double>(info, table);
    rc = gbdp_tabulate_fusion_se_a_grad_f64(gx.data_ptr<double>(), gm.data_ptr<double>(),
                                            table.data_ptr<double>(), hi.data(),
                                            em_x.data_ptr<double>(), em.data_ptr<double>(),
                                            dy.data_ptr<double>(), nloc, nnei, M, 1,
                                            cur_stream(table));
  } else {
    auto hi = host_info<float>(info, table);
    rc = gbdp_tabulate_fusion_se_a_grad_f32(gx.data_ptr<float>(), gm.data_ptr<float>(),
                                            table.data_ptr<float>(), hi.data(),
                                            em_x.data_ptr<float>(), em.data_ptr<float>(),
                                            dy.data_ptr<float>(), nloc, nnei, M, 1,
                                            cur_stream(table));
  }
  check_rc(rc, "tabulate_fusion_se_a_grad");
  return {gx, gm};
}

Tensor tab_grad_grad(const Tensor& table_in, const Tensor& info, const Tensor& em_x_in,
                     const Tensor& em_in, const Tensor& gx_in, const Tensor& gm_in, int64_t M) {
  const Tensor table = table_in.contiguous();
  const auto st = table.scalar_type();
  const Tensor em_x = em_x_in.to(st).contiguous();
  const Tensor em = em_in.to(st).contiguous();
  const Tensor gx = gx_in.to(st).contiguous();
  const Tensor gm = gm_in.to(st).contiguous();
  const int nloc = (int)em.size(0), nnei = (int)em.size(1);
  Tensor dz = torch::empty({nloc, 4, M}, table.options());
  int rc;
  if (st == torch::kFloat64) {
    auto hi = host_info<double>(info, table);
    rc = gbdp_tabulate_fusion_se_a_grad_grad_f64(
        dz.data_ptr<double>(), table.data_ptr<double>(), hi.data(), em_x.data_ptr<double>(),
        em.data_ptr<double>(), gx.data_ptr<double>(), gm.data_ptr<double>(), nloc, nnei, (int)M,
        1, cur_stream(table));
  } else {
    auto hi = host_info<float>(info, table);
    rc = gbdp_tabulate_fusion_se_a_grad_grad_f32(
        dz.data_ptr<float>(), table.data_ptr<float>(), hi.data(), em_x.data_ptr<float>(),
        em.data_ptr<float>(), gx.data_ptr<float>(), gm.data_ptr<float>(), nloc, nnei, (int)M, 1,
        cur_stream(table));
  }
  check_rc(rc, "tabulate_fusion_se_a_grad_grad");
  return dz;
}

// dy -> (dy_dem_x, dy_dem); differentiable wrt dy only (the grad-grad kernel)
struct TabGradFn : public torch::autograd::Function<TabGradFn> {
  static variable_list forward(AutogradContext* ctx, const Tensor& table, const Tensor& info,
                               const Tensor& em_x, const Tensor& em, const Tensor& dy) {
    ctx->save_for_backward({table, info, em_x, em});
    ctx->saved_data["M"] = dy.size(2);
    return tab_grad(table, info, em_x, em, dy);
  }
  static variable_list backward(AutogradContext* ctx, variable_list g) {
    auto s = ctx->get_saved_variables();
    Tensor gx = g[0].defined() ? g[0] : torch::zeros_like(s[2]);
    Tensor gm = g[1].defined() ? g[1] : torch::zeros_like(s[3]);
    Tensor dz = tab_grad_grad(s[0], s[1], s[2], s[3], gx, gm, ctx->saved_data["M"].toInt());
    return {Tensor(), Tensor(), Tensor(), Tensor(), dz};
  }
};

struct TabFn : public torch::autograd::Function<TabFn> {
  static Tensor forward(AutogradContext* ctx, const Tensor& table, const Tensor& info,
                        const Tensor& em_x, const Tensor& em, int64_t M) {
    ctx->save_for_backward({table, info, em_x, em});
    return tab_forward(table, info, em_x, em, M);
  }
  static variable_list backward(AutogradContext* ctx, variable_list g) {
    auto s = ctx->get_saved_variables();
    auto gg = TabGradFn::apply(s[0], s[1], s[2], s[3], g[0].contiguous());
    return {Tensor(), Tensor(), gg[0], gg[1], Tensor()};
  }
};

std::vector<Tensor> tabulate_fusion_se_a(const Tensor& table, const Tensor& table_info,
                                         const Tensor& em_x, const Tensor& em,
                                         int64_t last_layer_size) {
  return {TabFn::apply(table, table_info, em_x, em, last_layer_size)};
}

Tensor enable_mpi() { return torch::zeros({1}, torch::kBool); }

}  // namespace

TORCH_LIBRARY(deepmd, m) {
  m.def("enable_mpi", enable_mpi);
  m.def("tabulate_fusion_se_a", tabulate_fusion_se_a);
}
