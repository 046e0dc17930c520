// mfc_gpu_tvd_rk_noalloc: one TVD-RK time step that allocates nothing.
//
// Who needs it: hosts that cannot call cudaMalloc/cudaFree from the solver
// step.  Examples are hosts whose device memory is owned by another
// allocator (a framework's caching pool, or an OpenACC runtime whose
// present table owns the state arrays and that hands their device addresses
// over with `host_data use_device`), which must not see foreign allocations
// appear or fail under their memory budget, and hosts that must not trigger
// the device-wide synchronisation that cudaMalloc/cudaFree can cause in the
// middle of their own stream work.  The regular entry points allocate their
// RK registers and grid tables once, in mfc_gpu_init; this one instead uses
// the file-scope device array below.
//
// The caller passes the state at t^n (q_in) and receives the state at
// t^{n+1} (q_out), both device arrays of doubles laid out [S][p+1][n+1][ld_y]
// (x fastest).  The one intermediate RK register, the grid tables and the
// status word live in g_noalloc_scratch, whose size is fixed at compile time:
//   - S * (n+1) * (p+1) * ld_y  <= kNoAllocMaxRegElems (7 * 2^20 doubles,
//     e.g. 1024 x 1024 cells of the 7-equation 2-D model),
//   - at most kNoAllocMaxCells cells per direction (4096),
// about 58 MiB that every GPU which loads this library keeps until the
// process exits.  Larger cases are rejected with MFC_ERR_INVALID.
//
// Every call shares the array and overwrites what the previous call left in
// it (the status word is cleared at the start of each call; the register and
// tables are fully rewritten before they are read).  Calls that overlap on
// the GPU -- concurrent calls on different streams or host threads -- race
// on the array.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture.  The call is synchronous with respect to
// `stream`.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mfc_gpu.h"
#include "mfc_grid.h"
#include "mfc_launch.h"

namespace {

constexpr int64_t kNoAllocMaxRegElems = int64_t(7) << 20;
constexpr int kNoAllocMaxCells = 4096;
// per direction: 1/dx of the cells, the cell-centre spacings (cells + 1) and
// the coefficient rows (cells + 2 * kCoefPad each), as build_grid_tables
// lays them out
constexpr int64_t kNoAllocTableElems =
    3 * (int64_t(kNoAllocMaxCells) + (int64_t(kNoAllocMaxCells) + 1) +
         int64_t(mfc::kNumCoef) * (kNoAllocMaxCells + 2 * mfc::kCoefPad));
constexpr int64_t kNoAllocStatusOffset = kNoAllocMaxRegElems + kNoAllocTableElems;
constexpr int64_t kNoAllocScratchElems = kNoAllocStatusOffset + 32;  // + one 256-byte slot for the status word

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (which must be current),
// looked up once per device.
cudaError_t scratch_address(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[device]) {
    double* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = ptr;
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

struct DeviceGuard {
  int prev = -1;
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" int mfc_gpu_tvd_rk_noalloc(const mfc_params* p, const double* q_in, double* q_out, int64_t ld_y,
                                      double dt, void* stream) {
  const std::string why = mfc::validate_params(p);
  if (!why.empty()) return mfc::report_error(MFC_ERR_INVALID, why);
  if (p->p > 0)
    return mfc::report_error(MFC_ERR_INVALID, "mfc_gpu_tvd_rk_noalloc handles 1-D and 2-D cases; 3-D cases need "
                                              "the RHS work buffer that mfc_gpu_init allocates");
  if (p->precision == MFC_PREC_GATED)
    return mfc::report_error(MFC_ERR_INVALID, "mfc_gpu_tvd_rk_noalloc takes MFC_PREC_FP64 or MFC_PREC_SPLIT; the "
                                              "learned gate needs the parameters that mfc_gpu_set_gate uploads");
  if (!q_in || !q_out) return mfc::report_error(MFC_ERR_INVALID, "q_in and q_out must be device arrays");
  if (q_in == q_out) return mfc::report_error(MFC_ERR_INVALID, "q_in and q_out must be different arrays");
  const int nd = 1 + (p->n > 0) + (p->p > 0);
  const int S = 2 * p->num_fluids + nd + 1;
  const int n[3] = {p->m + 1, p->n + 1, p->p + 1};
  if (ld_y < n[0]) return mfc::report_error(MFC_ERR_INVALID, "ld_y is smaller than m+1");
  for (int d = 0; d < nd; ++d)
    if (n[d] > kNoAllocMaxCells)
      return mfc::report_error(MFC_ERR_INVALID, "mfc_gpu_tvd_rk_noalloc: more than 4096 cells in a direction "
                                                "exceeds its fixed scratch; use mfc_gpu_init/mfc_gpu_tvd_rk");
  const int64_t sz = ld_y * n[1], sv = sz * n[2];
  if (sv * S > kNoAllocMaxRegElems)
    return mfc::report_error(MFC_ERR_INVALID, "mfc_gpu_tvd_rk_noalloc: S*(n+1)*(p+1)*ld_y exceeds its fixed scratch "
                                              "of 7*2^20 doubles; use mfc_gpu_init/mfc_gpu_tvd_rk");
  if (p->device < 0 || p->device >= kMaxDevices) return mfc::report_error(MFC_ERR_INVALID, "device out of range");
  const mfc::StageEntry* stage = mfc::find_stage(nd, p->num_fluids, p->weno_order, p->precision);
  if (!stage) return mfc::report_error(MFC_ERR_INVALID, "no kernel compiled for this configuration");

  const int b = (p->weno_order - 1) / 2 + 2;
  mfc::GridTables gt;
  const std::string gwhy = mfc::build_grid_tables(p, nd, n, b, gt);
  if (!gwhy.empty()) return mfc::report_error(MFC_ERR_INVALID, gwhy);
  if ((int64_t)gt.host.size() > kNoAllocTableElems)
    return mfc::report_error(MFC_ERR_INVALID, "mfc_gpu_tvd_rk_noalloc: the grid tables exceed their fixed scratch");

  DeviceGuard guard;
  cudaError_t e = cudaGetDevice(&guard.prev);
  if (e == cudaSuccess && guard.prev != p->device) e = cudaSetDevice(p->device);
  double* scratch = nullptr;
  if (e == cudaSuccess) e = scratch_address(p->device, &scratch);
  if (e != cudaSuccess) return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* reg = scratch;
  double* tables = scratch + kNoAllocMaxRegElems;
  uint32_t* status = reinterpret_cast<uint32_t*>(scratch + kNoAllocStatusOffset);

  mfc::DevParams D{};
  const int bcb[3] = {p->bc_x_beg, p->bc_y_beg, p->bc_z_beg};
  const int bce[3] = {p->bc_x_end, p->bc_y_end, p->bc_z_end};
  for (int d = 0; d < 3; ++d) {
    D.n[d] = n[d];
    D.bc_beg[d] = bcb[d];
    D.bc_end[d] = bce[d];
    D.inv_d[d] = d < nd ? tables + gt.off_inv[d] : nullptr;
    D.coef[d] = d < nd ? tables + gt.off_coef[d] : nullptr;
    D.cstride[d] = gt.cstride[d];
  }
  D.sy = ld_y;
  D.sz = sz;
  D.sv = sv;
  for (int f = 0; f < mfc::kMaxFluids; ++f) {
    D.gammas[f] = f < p->num_fluids ? p->gammas[f] : 0.0;
    D.pi_infs[f] = f < p->num_fluids ? p->pi_infs[f] : 0.0;
  }
  D.weno_eps = p->weno_eps;
  mfc::set_fp32_constants(D);
  D.coff = mfc::kCoefPad;
  D.status = status;
  mfc::UniformCoef U;
  mfc::uniform_records(gt, nd, n, p->weno_order, p->precision, U);

  if ((e = stage->prepare()) != cudaSuccess) return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaMemcpyAsync(tables, gt.host.data(), sizeof(double) * gt.host.size(), cudaMemcpyHostToDevice, st)) !=
      cudaSuccess)
    return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st)) != cudaSuccess)
    return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));

  // RK3: q_in -> q_out -> reg -> q_out; RK2: q_in -> reg -> q_out; RK1: q_in -> q_out.
  // A stage never writes the register it reads its halo from.
  switch (p->time_stepper) {
    case 1:
      e = stage->launch(D, U, q_in, q_in, q_out, dt, mfc::kRkEuler, st);
      break;
    case 2:
      e = stage->launch(D, U, q_in, q_in, reg, dt, mfc::kRkEuler, st);
      if (e == cudaSuccess) e = stage->launch(D, U, reg, q_in, q_out, dt, mfc::kRk2Final, st);
      break;
    default:
      e = stage->launch(D, U, q_in, q_in, q_out, dt, mfc::kRkEuler, st);
      if (e == cudaSuccess) e = stage->launch(D, U, q_out, q_in, reg, dt, mfc::kRk3Mid, st);
      if (e == cudaSuccess) e = stage->launch(D, U, reg, q_in, q_out, dt, mfc::kRk3Final, st);
      break;
  }
  if (e != cudaSuccess) return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  uint32_t flags = 0;
  if ((e = cudaMemcpyAsync(&flags, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return mfc::report_error(MFC_ERR_CUDA, cudaGetErrorString(e));
  if (flags & MFC_FLAG_NAN) return mfc::report_error(MFC_ERR_STATE, "NaN or Inf in the conservative state");
  if (flags & MFC_FLAG_TIMEOUT)
    return mfc::report_error(MFC_ERR_STATE, "a TMA staging wait timed out; tiles of q_out were not written");
  return MFC_OK;
}
