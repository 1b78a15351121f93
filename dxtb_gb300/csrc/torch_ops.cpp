// torch operators over the C ABI of libgbxtb.so (namespace gbxtb).
//
//   gbxtb::singlepoint(int plan, Tensor positions, Tensor workspace,
//                      int[] iopts, float[] fopts)
//       -> (Tensor energy, Tensor charges, Tensor state, Tensor status)
//   gbxtb::forces_backward(Tensor state, Tensor grad_energy, Tensor atom_mol)
//       -> Tensor
//
// `plan` is a gbxtb_plan handle (gbxtb_plan_create), which fixes the
// molecules' atomic numbers, charges and spins; `positions` are the ragged
// positions of its atoms ([natoms][3], bohr, float64, CUDA) and `workspace`
// a byte tensor of at least the plan's workspace size on the same device.
// The call runs gbxtb_singlepoint on torch's current stream of that device
// and returns the energy per molecule (nmol), the Mulliken atomic charges
// (natoms), the state of the adjoint (the gradient dE/dR, [natoms][3]; an
// empty tensor unless iopts asks for forces) and, on the host, the status
// bits and SCF iteration counts per molecule ([nmol][2], int32).
// forces_backward contracts that state with the incoming gradient of the
// energies: dL/dR_a = dL/dE_{mol(a)} dE/dR_a, atom_mol mapping atoms to
// molecules.  Together they are the reference's differentiable single point
// (calculators/types/energy.py:78-402 forward, types/autograd.py:82-201
// backward), wrapped by dxtb_gb300.calculator's autograd Function.
//
// iopts: maxiter, fermi_maxiter, broyden_memory, want_forces, profile,
//        mixed_precision, mixer, generations, soft_start, mix_guess,
//        damp_dynamic, no_halogen, restart_at, fp64_split
// fopts: x_atol, x_atol_max, kt, broyden_alpha, damp, damp_init,
//        diagonal_offset, damp_dynamic_factor, fermi_thresh
#include <ATen/ATen.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/library.h>

#include <string>
#include <vector>

#include "gbxtb.h"

namespace {

constexpr size_t kIopts = 14, kFopts = 9;

gbxtb_options unpack_options(const std::vector<int64_t> &io, const std::vector<double> &fo) {
  TORCH_CHECK(io.size() == kIopts, "gbxtb::singlepoint: iopts needs ", kIopts, " entries, got ", io.size());
  TORCH_CHECK(fo.size() == kFopts, "gbxtb::singlepoint: fopts needs ", kFopts, " entries, got ", fo.size());
  gbxtb_options o;
  gbxtb_default_options(&o);
  o.maxiter = (int32_t)io[0];
  o.fermi_maxiter = (int32_t)io[1];
  o.broyden_memory = (int32_t)io[2];
  o.want_forces = (int32_t)io[3];
  o.profile = (int32_t)io[4];
  o.mixed_precision = (int32_t)io[5];
  o.mixer = (int32_t)io[6];
  o.generations = (int32_t)io[7];
  o.soft_start = (int32_t)io[8];
  o.mix_guess = (int32_t)io[9];
  o.damp_dynamic = (int32_t)io[10];
  o.no_halogen = (int32_t)io[11];
  o.restart_at = (int32_t)io[12];
  o.fp64_split = (int32_t)io[13];
  o.x_atol = fo[0];
  o.x_atol_max = fo[1];
  o.kt = fo[2];
  o.broyden_alpha = fo[3];
  o.damp = fo[4];
  o.damp_init = fo[5];
  o.diagonal_offset = fo[6];
  o.damp_dynamic_factor = fo[7];
  o.fermi_thresh = fo[8];
  return o;
}

void check_rc(int rc, const char *what) {
  TORCH_CHECK(rc == GBXTB_OK, what, " failed (gbxtb error ", rc, "): ", gbxtb_last_error());
}

std::tuple<at::Tensor, at::Tensor, at::Tensor, at::Tensor> singlepoint(int64_t plan_handle,
                                                                       const at::Tensor &positions,
                                                                       const at::Tensor &workspace,
                                                                       at::IntArrayRef iopts,
                                                                       at::ArrayRef<double> fopts) {
  auto *plan = reinterpret_cast<gbxtb_plan *>(plan_handle);
  TORCH_CHECK(plan != nullptr, "gbxtb::singlepoint: null plan");
  int64_t sizes[6];
  check_rc(gbxtb_plan_sizes(plan, sizes), "gbxtb_plan_sizes");
  const int64_t nmol = sizes[0], natom = sizes[1];
  TORCH_CHECK(positions.is_cuda() && positions.scalar_type() == at::kDouble,
              "gbxtb::singlepoint: positions must be a float64 CUDA tensor");
  TORCH_CHECK(positions.dim() == 2 && positions.size(0) == natom && positions.size(1) == 3,
              "gbxtb::singlepoint: positions must have shape (", natom, ", 3), got ", positions.sizes());
  TORCH_CHECK(workspace.is_cuda() && workspace.device() == positions.device() && workspace.is_contiguous(),
              "gbxtb::singlepoint: workspace must be a contiguous tensor on the device of the positions");
  const gbxtb_options opts =
      unpack_options(std::vector<int64_t>(iopts.begin(), iopts.end()), std::vector<double>(fopts.begin(), fopts.end()));
  const c10::cuda::CUDAGuard guard(positions.device());
  const at::Tensor pos = positions.contiguous();
  const auto f64 = positions.options();
  at::Tensor energy = at::empty({nmol}, f64);
  at::Tensor charges = at::empty({natom}, f64);
  at::Tensor state = opts.want_forces ? at::empty({natom, 3}, f64) : at::empty({0}, f64);
  cudaStream_t stream = c10::cuda::getCurrentCUDAStream(positions.device().index()).stream();
  check_rc(gbxtb_singlepoint(plan, &opts, pos.data_ptr<double>(), energy.data_ptr<double>(),
                             charges.data_ptr<double>(), opts.want_forces ? state.data_ptr<double>() : nullptr,
                             workspace.data_ptr(), (size_t)workspace.nbytes(), stream),
           "gbxtb_singlepoint");
  at::Tensor status = at::empty({nmol, 2}, at::TensorOptions().dtype(at::kInt));
  std::vector<int32_t> st(nmol), it(nmol);
  check_rc(gbxtb_get_status(plan, st.data(), it.data()), "gbxtb_get_status");
  int32_t *sp = status.data_ptr<int32_t>();
  for (int64_t m = 0; m < nmol; ++m) {
    sp[2 * m] = st[m];
    sp[2 * m + 1] = it[m];
  }
  return {energy, charges, state, status};
}

at::Tensor forces_backward(const at::Tensor &state, const at::Tensor &grad_energy, const at::Tensor &atom_mol) {
  TORCH_CHECK(state.dim() == 2 && state.size(1) == 3, "gbxtb::forces_backward: state must be (natoms, 3)");
  TORCH_CHECK(atom_mol.dim() == 1 && atom_mol.size(0) == state.size(0),
              "gbxtb::forces_backward: atom_mol must have one entry per atom");
  const at::Tensor g = grad_energy.reshape({-1}).to(state.options());
  return g.index_select(0, atom_mol.to(state.device(), at::kLong)).unsqueeze(-1) * state;
}

}  // namespace

TORCH_LIBRARY(gbxtb, m) {
  m.def("singlepoint(int plan, Tensor positions, Tensor workspace, int[] iopts, float[] fopts) -> "
        "(Tensor energy, Tensor charges, Tensor state, Tensor status)");
  m.def("forces_backward(Tensor state, Tensor grad_energy, Tensor atom_mol) -> Tensor");
}

TORCH_LIBRARY_IMPL(gbxtb, CUDA, m) {
  m.impl("singlepoint", &singlepoint);
  m.impl("forces_backward", &forces_backward);
}
