// engine.cu -- the box handle API: device-resident time stepping with the time step kept on
// the device, optional CUDA-graph replay, and per-kernel timing.
//
// One cgb_box owns the scratch of one padded box, so boxes of different sizes coexist in
// one process (the reference keeps its scratch in file-scope globals and static launch
// parameters, src/global/global_cuda.cu:1-16, VL_3D_cuda.cu:141).  One call advances a box
// by n steps with no host synchronisation: ghost fill -> dt = C_cfl / max_dti (clamped to
// t_end) -> predictor -> corrector -> finalize (DE select/sync, temperature floor, CFL
// reduction for the next step), i.e. the body of the reference's main loop
// (src/main.cpp:247-379) for one box.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cholla_gb300.h"
#include "common.cuh"
#include "kernels.h"

struct cgb_box {
  cgb::Box b;
  cgb_scheme scheme;
  int flags[6];
  cgb::Scratch s{};
  double *dt_t = nullptr;  // device [dt, t]
  double t_end = 0.0;
  bool dti_valid = false;
  // graph of one step (captured on first use per state pointer, stream and CFL number)
  cudaGraphExec_t graph = nullptr;
  double *graph_U = nullptr;
  cudaStream_t graph_stream = nullptr;
  double graph_cfl = 0.0;  // the CFL number is baked into the captured dt launch
  bool use_graph = false;
  // timing: four events per timed step (before predictor, after predictor, after corrector,
  // after finalize), recorded on the launching stream and read back by cgb_box_kernel_times
  bool timing = false;
  std::vector<cudaEvent_t> marks;
  size_t used = 0;
  double ms[3] = {0, 0, 0};
  long long launches = 0;
  cudaStream_t last_stream = nullptr;
  std::string err;
};

namespace
{
thread_local std::string g_box_err;

int box_fail(cgb_box *bx, int code, const std::string &m)
{
  if (bx) bx->err = m;
  g_box_err = m;
  return code;
}

void free_box_mem(cgb_box *bx)
{
  void *ps[] = {bx->s.Uh, bx->s.GEp, bx->s.Epre, bx->s.emf, bx->s.Fx, bx->s.Fy, bx->s.Fz, bx->s.dti, bx->s.status,
                bx->dt_t, bx->s.W, bx->s.mhd};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (bx->graph) cudaGraphExecDestroy(bx->graph);
  for (auto &e : bx->marks)
    if (e) cudaEventDestroy(e);
  bx->marks.clear();
}

// fold the recorded events into the per-kernel sums
cudaError_t collect_times(cgb_box *bx)
{
  for (size_t i = 0; i + 3 < bx->used; i += 4) {
    cudaError_t e = cudaEventSynchronize(bx->marks[i + 3]);
    if (e != cudaSuccess) return e;
    float a = 0, c = 0, f = 0;
    cudaEventElapsedTime(&a, bx->marks[i], bx->marks[i + 1]);
    cudaEventElapsedTime(&c, bx->marks[i + 1], bx->marks[i + 2]);
    cudaEventElapsedTime(&f, bx->marks[i + 2], bx->marks[i + 3]);
    bx->ms[0] += a, bx->ms[1] += c, bx->ms[2] += f;
    bx->launches++;
  }
  bx->used = 0;
  return cudaSuccess;
}

cudaError_t one_step(cgb_box *bx, double *U, double c_cfl, cudaStream_t st, bool timed)
{
  cudaError_t e = cgb::set_boundaries(bx->b, U, bx->flags, st);
  if (e != cudaSuccess) return e;
  if ((e = cgb::cfl_dt(bx->s.dti, bx->dt_t, c_cfl, bx->t_end, st)) != cudaSuccess) return e;
  cudaEvent_t *m = nullptr;
  if (timed) {
    if (bx->used + 4 > bx->marks.size()) {
      if ((e = collect_times(bx)) != cudaSuccess) return e;
      while (bx->marks.size() < 4 * 64) {
        cudaEvent_t ev;
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return e;
        bx->marks.push_back(ev);
      }
    }
    m = &bx->marks[bx->used];
    bx->used += 4;
  }
  if (bx->b.mhd) {
    // MHD: the step, the temperature floor, then the CFL reduction for the next step (the
    // fast magnetosonic speed needs the cell-centred field, so it is its own pass)
    if (m) cudaEventRecord(m[0], st);
    if ((e = cgb::mhd_step(bx->b, bx->scheme.reconstruction, bx->scheme.precision, U, bx->s.mhd, 0.0, bx->dt_t, st)) !=
        cudaSuccess)
      return e;
    if (m) cudaEventRecord(m[1], st), cudaEventRecord(m[2], st);
    if (bx->scheme.temperature_floor &&
        (e = cgb::hydro_temperature_floor(bx->b, U, bx->scheme.U_floor, st)) != cudaSuccess)
      return e;
    if ((e = cgb::mhd_calc_dt(bx->b, U, bx->s.dti, st)) != cudaSuccess) return e;
    if (m) cudaEventRecord(m[3], st);
    return cudaSuccess;
  }
  return cgb::hydro_step(bx->b, bx->scheme.reconstruction, bx->scheme.riemann_solver, bx->scheme.precision, U, bx->s,
                         0.0, bx->dt_t, bx->scheme.U_floor, bx->scheme.temperature_floor, 1, st, m, 1);
}
}  // namespace

extern "C" {

const char *cgb_box_last_error(void) { return g_box_err.c_str(); }

int cgb_box_create(cgb_box **out, int nx, int ny, int nz, int n_ghost, double dx, double dy, double dz,
                   const cgb_scheme *scheme, const int flags[6])
{
  if (!out || !scheme || !flags) return box_fail(nullptr, CGB_ERR_ARGS, "null argument");
  *out = nullptr;
  cgb_scheme const &s = *scheme;
  if (s.reconstruction < CGB_PCM || s.reconstruction > CGB_PPMP || s.riemann_solver < CGB_HLLC ||
      s.riemann_solver > CGB_EXACT)
    return box_fail(nullptr, CGB_ERR_ARGS, "bad reconstruction or riemann solver");
  if (s.precision < CGB_FP64 || s.precision > CGB_FP64_FAST) return box_fail(nullptr, CGB_ERR_ARGS, "bad precision");
  if (s.n_scalars < 0 || s.n_scalars > cgb::NS_MAX || !(s.gamma > 1.0) || (s.riemann_solver == CGB_HLLD) != (s.mhd != 0))
    return box_fail(nullptr, CGB_ERR_ARGS, "bad scheme (MHD goes with HLLD and only with it)");
  if (s.mhd && (s.precision == CGB_MIXED || s.dual_energy || ny < 2 || nz < 2))
    return box_fail(nullptr, CGB_ERR_UNSUPPORTED, "MHD boxes are 3D, exact or fast FP64, without dual energy");
  bool const one_d = ny == 1 && nz == 1, two_d = nz == 1 && ny > 1;
  if ((one_d || two_d) && s.riemann_solver == CGB_HLL)
    return box_fail(nullptr, CGB_ERR_UNSUPPORTED, "the reference's 1D and 2D integrators have no HLL branch");
  if (two_d && (s.precision != CGB_FP64 || s.mhd))
    return box_fail(nullptr, CGB_ERR_UNSUPPORTED, "2D boxes are hydro, exact FP64 form only");
  int const H = (s.reconstruction == CGB_PPMC || s.reconstruction == CGB_PPMP   ? 4
                 : s.reconstruction == CGB_PLMC || s.reconstruction == CGB_PLMP ? 3
                                                                                : 2) +
                (s.mhd ? 1 : 0);
  if (n_ghost < H || nx < 2 * n_ghost + 1 ||
      (!one_d && (ny < 2 * n_ghost + 1 || (!two_d && nz < 2 * n_ghost + 1))))
    return box_fail(nullptr, CGB_ERR_ARGS, "box too small for the reconstruction stencil");
  if (!(dx > 0 && dy > 0 && dz > 0)) return box_fail(nullptr, CGB_ERR_ARGS, "cell sizes must be positive");
  for (int i = 0; i < 6; i++)
    if (flags[i] < 0 || flags[i] > 5) return box_fail(nullptr, CGB_ERR_ARGS, "boundary flags must be 0..5");
  cgb_box *bx = new cgb_box();
  bx->scheme  = s;
  std::memcpy(bx->flags, flags, sizeof(bx->flags));
  cgb::Box &b = bx->b;
  b.nx = nx, b.ny = ny, b.nz = nz, b.ng = n_ghost, b.ns = s.n_scalars;
  b.de = s.dual_energy ? 1 : 0, b.mhd = s.mhd ? 1 : 0;
  b.nf = 5 + s.n_scalars + b.de + 3 * b.mhd;
  b.floor_on = (one_d || two_d) ? 0 : (s.density_floor ? 1 : 0);  // the 1D and 2D updates have no density floor
  b.n = (long long)nx * ny * nz;
  b.gamma = s.gamma, b.dx = dx, b.dy = dy, b.dz = dz, b.density_floor = 0.0;
  size_t const n = (size_t)b.n;
  auto al = [](void **p, size_t bytes) {
    if (cgb::dev_malloc(p, bytes) != cudaSuccess) return false;
    return cudaMemset(*p, 0, bytes) == cudaSuccess;
  };
  bool ok = al((void **)&bx->s.dti, 8) && al((void **)&bx->s.status, 8) && al((void **)&bx->dt_t, 16);
  if (ok && b.mhd) {
    ok = al((void **)&bx->s.mhd, cgb::mhd_scratch_doubles(b) * 8);
  } else if (ok) {
    ok = al((void **)&bx->s.Uh, n * b.nf * 8) && al((void **)&bx->s.GEp, n * 8) && al((void **)&bx->s.Epre, n * 8) &&
         al((void **)&bx->s.W, 2 * (size_t)(b.nf + 1) * n * 8);
  }
  if (!ok) {
    cudaGetLastError();
    free_box_mem(bx);
    delete bx;
    return box_fail(nullptr, CGB_ERR_NOMEM, "box scratch allocation failed");
  }
  *out = bx;
  return CGB_OK;
}

int cgb_box_destroy(cgb_box *bx)
{
  if (!bx) return CGB_OK;
  if (bx->last_stream) cudaStreamSynchronize(bx->last_stream);
  free_box_mem(bx);
  delete bx;
  return CGB_OK;
}

int cgb_box_n_fields(const cgb_box *bx) { return bx ? bx->b.nf : -1; }

int cgb_box_set_time(cgb_box *bx, double t, double t_end)
{
  if (!bx) return box_fail(nullptr, CGB_ERR_ARGS, "null box");
  double h[2] = {0.0, t};
  // steps still queued on the box's stream read [dt, t]: let them finish before it is replaced
  if (cudaStreamSynchronize(bx->last_stream) != cudaSuccess ||
      cudaMemcpy(bx->dt_t, h, 16, cudaMemcpyHostToDevice) != cudaSuccess)
    return box_fail(bx, CGB_ERR_CUDA, "set_time copy");
  bx->t_end = t_end;
  if (bx->graph) {  // t_end is baked into the captured launch
    cudaGraphExecDestroy(bx->graph);
    bx->graph = nullptr;
  }
  return CGB_OK;
}

int cgb_box_use_graph(cgb_box *bx, int enable)
{
  if (!bx) return box_fail(nullptr, CGB_ERR_ARGS, "null box");
  bx->use_graph = enable != 0;
  return CGB_OK;
}

int cgb_box_enable_timing(cgb_box *bx, int enable)
{
  if (!bx) return box_fail(nullptr, CGB_ERR_ARGS, "null box");
  bx->timing = enable != 0;
  bx->used   = 0;
  bx->ms[0] = bx->ms[1] = bx->ms[2] = 0.0;
  bx->launches = 0;
  return CGB_OK;
}

// ms[0] predictor, ms[1] corrector, ms[2] finalize (incl. negative-density pass); summed over
// the timed steps; *steps = number of timed steps.
int cgb_box_kernel_times(cgb_box *bx, double ms[3], long long *steps)
{
  if (!bx || !ms || !steps) return box_fail(bx, CGB_ERR_ARGS, "null argument");
  cudaError_t e = collect_times(bx);
  if (e != cudaSuccess) return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
  for (int i = 0; i < 3; i++) ms[i] = bx->ms[i];
  *steps = bx->launches;
  return CGB_OK;
}

// Advance the box by n_steps on `stream` (cudaStream_t, NULL = legacy default stream) with
// dt = c_cfl / max_dti from the previous reduction.  No host synchronisation unless timing
// is enabled.  d_conserved is updated in place; its ghost cells are refilled first.
int cgb_box_advance(cgb_box *bx, double *d_conserved, int n_steps, double c_cfl, void *stream)
{
  if (!bx || !d_conserved || n_steps < 0 || !(c_cfl > 0)) return box_fail(bx, CGB_ERR_ARGS, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  bx->last_stream = st;
  cudaError_t e;
  if (!bx->dti_valid) {
    if ((e = bx->b.mhd ? cgb::mhd_calc_dt(bx->b, d_conserved, bx->s.dti, st)
                       : cgb::hydro_calc_dt(bx->b, d_conserved, bx->s.dti, st)) != cudaSuccess)
      return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
    bx->dti_valid = true;
  }
  // the state may have changed since the last call: the first step forms every cell's primitives
  // (status[1], the fast forms' carried-primitives flag, set again by each step's finalize)
  if (!bx->b.mhd && (e = cudaMemsetAsync(bx->s.status + 1, 0, sizeof(int), st)) != cudaSuccess)
    return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
  bool const graph_ok = bx->use_graph && !bx->timing && st != nullptr;
  if (graph_ok && (!bx->graph || bx->graph_U != d_conserved || bx->graph_stream != st || bx->graph_cfl != c_cfl)) {
    if (bx->graph) cudaGraphExecDestroy(bx->graph), bx->graph = nullptr;
    cudaGraph_t g;
    if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
    cudaError_t ce = one_step(bx, d_conserved, c_cfl, st, false);
    e              = cudaStreamEndCapture(st, &g);
    if (ce != cudaSuccess || e != cudaSuccess)
      return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(ce != cudaSuccess ? ce : e));
    e = cudaGraphInstantiate(&bx->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
    bx->graph_U      = d_conserved;
    bx->graph_stream = st;
    bx->graph_cfl    = c_cfl;
  }
  for (int i = 0; i < n_steps; i++) {
    if (graph_ok) {
      e = cudaGraphLaunch(bx->graph, st);
    } else {
      e = one_step(bx, d_conserved, c_cfl, st, bx->timing);
    }
    if (e != cudaSuccess) return box_fail(bx, CGB_ERR_CUDA, cudaGetErrorString(e));
  }
  return CGB_OK;
}

namespace
{
const char *kBadCells =
    "the box holds a real cell with non-finite density or energy, or density <= 0 after the negative-density repair";
const char *kTimeout = "a bounded device wait for a TMA copy ran out; a step left a tile undone";
}

// Current (dt, t) of the box; synchronises the box's last stream.  Returns CGB_ERR_NONFINITE (with
// t and dt filled in) while the box's status word records a bad cell.
int cgb_box_get_time(cgb_box *bx, double *t, double *dt_last)
{
  if (!bx) return box_fail(nullptr, CGB_ERR_ARGS, "null box");
  double h[2];
  int st = 0;
  if (cudaStreamSynchronize(bx->last_stream) != cudaSuccess ||
      cudaMemcpy(h, bx->dt_t, 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&st, bx->s.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return box_fail(bx, CGB_ERR_CUDA, "get_time");
  if (dt_last) *dt_last = h[0];
  if (t) *t = h[1];
  if (st & CGB_STATUS_TIMEOUT) return box_fail(bx, CGB_ERR_TIMEOUT, kTimeout);
  if (st & CGB_STATUS_NONFINITE) return box_fail(bx, CGB_ERR_NONFINITE, kBadCells);
  return CGB_OK;
}

// The box's status bits (CGB_STATUS_*) since the last call, which clears them; synchronises the
// box's last stream.  CGB_ERR_NONFINITE when CGB_STATUS_NONFINITE is among them.
int cgb_box_check_status(cgb_box *bx, int *flags)
{
  if (!bx) return box_fail(nullptr, CGB_ERR_ARGS, "null box");
  int st = 0;
  if (cudaStreamSynchronize(bx->last_stream) != cudaSuccess ||
      cudaMemcpy(&st, bx->s.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemset(bx->s.status, 0, sizeof(int)) != cudaSuccess)
    return box_fail(bx, CGB_ERR_CUDA, "check_status");
  if (flags) *flags = st;
  if (st & CGB_STATUS_TIMEOUT) return box_fail(bx, CGB_ERR_TIMEOUT, kTimeout);
  if (st & CGB_STATUS_NONFINITE) return box_fail(bx, CGB_ERR_NONFINITE, kBadCells);
  return CGB_OK;
}

}  // extern "C"
