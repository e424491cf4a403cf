// capi.cu -- the C ABI of libchollagb (declared in include/cholla_gb300.h).
//
// Host-side bookkeeping only: argument checks, the run-time scheme, per-shape scratch and
// kernel dispatch.  No entry point falls back to host computation: if a kernel cannot run
// the call returns an error.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/cholla_gb300.h"
#include "common.cuh"
#include "kernels.h"

namespace
{
std::mutex g_mu;
cgb_scheme g_scheme = {CGB_PPMC, CGB_HLLC, 1, 0, 0, 1, 1, CGB_FP64, 5.0 / 3.0, 0.0};
cudaStream_t g_stream = nullptr;
thread_local std::string g_err;

struct ScratchSlot {
  int nx = 0, ny = 0, nz = 0, nf = 0, mhd = -1;
  int dev = -1;  // device the scratch was allocated on
  cgb::Scratch s{};
  bool live = false;
};
ScratchSlot g_slot;
// Reductions the drop-in calls return (max inverse dt, max |div B|) come back through one word of
// mapped pinned memory that a one-thread kernel writes, not through a device-to-host copy: a copy
// waits on the copy engine behind every large transfer queued before it, so a caller that overlaps
// its state uploads and downloads with the steps would stall for them at every dt readback.
unsigned long long *g_word_host = nullptr;           // mapped pinned word (host address)
unsigned long long *g_word_dev  = nullptr;           // its device address
__global__ void k_put_word(const unsigned long long *__restrict__ src, unsigned long long *dst) { *dst = *src; }

int fail(int code, const std::string &msg)
{
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *where)
{
  return fail(CGB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// the word at d_src, read on the host after the drop-in stream reaches it
int read_word(const unsigned long long *d_src, unsigned long long *out, const char *where)
{
  if (!g_word_host) {
    if (cudaHostAlloc((void **)&g_word_host, sizeof(unsigned long long), cudaHostAllocMapped | cudaHostAllocPortable) !=
        cudaSuccess) {
      g_word_host = nullptr;
      return fail(CGB_ERR_NOMEM, "pinned result word");
    }
    if (cudaHostGetDevicePointer((void **)&g_word_dev, g_word_host, 0) != cudaSuccess) {
      cudaFreeHost(g_word_host);
      g_word_host = nullptr;
      return fail(CGB_ERR_CUDA, "mapped result word");
    }
  }
  k_put_word<<<1, 1, 0, g_stream>>>(d_src, g_word_dev);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_stream);
  if (e != cudaSuccess) return cuda_fail(e, where);
  *out = *(volatile unsigned long long *)g_word_host;
  return CGB_OK;
}

void free_slot(ScratchSlot &sl)
{
  if (!sl.live) return;
  int cur = -1;
  bool const other = cudaGetDevice(&cur) == cudaSuccess && sl.dev >= 0 && sl.dev != cur;
  if (other) cudaSetDevice(sl.dev);  // free on the device that owns the scratch
  cudaFree(sl.s.Uh);
  cudaFree(sl.s.GEp);
  cudaFree(sl.s.Epre);
  cudaFree(sl.s.emf);
  cudaFree(sl.s.Fx);
  cudaFree(sl.s.Fy);
  cudaFree(sl.s.Fz);
  cudaFree(sl.s.dti);
  cudaFree(sl.s.status);
  cudaFree(sl.s.W);
  cudaFree(sl.s.mhd);
  if (other) cudaSetDevice(cur);
  sl = ScratchSlot{};
}

int ensure_slot(int nx, int ny, int nz, int nf, int mhd)
{
  int dev       = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (g_slot.live && g_slot.nx == nx && g_slot.ny == ny && g_slot.nz == nz && g_slot.nf == nf &&
      g_slot.mhd == mhd && g_slot.dev == dev)
    return CGB_OK;
  free_slot(g_slot);
  size_t const n = (size_t)nx * ny * nz;
  cgb::Scratch s{};
  auto alloc = [&](void **p, size_t bytes) -> bool {
    if (bytes == 0) {
      *p = nullptr;
      return true;
    }
    if (cgb::dev_malloc(p, bytes) != cudaSuccess) return false;
    return cudaMemset(*p, 0, bytes) == cudaSuccess;
  };
  bool ok = alloc((void **)&s.dti, sizeof(unsigned long long)) && alloc((void **)&s.status, sizeof(int));
  if (ok && mhd) {
    // U½ + 6 interface-state arrays + 3 flux arrays of nf - 1 fields + 3 EMF fields
    ok = alloc((void **)&s.mhd, cgb::mhd_scratch_fields(nf) * n * sizeof(double));
  } else if (ok) {
    ok = alloc((void **)&s.Uh, n * nf * sizeof(double)) && alloc((void **)&s.GEp, n * sizeof(double)) &&
         alloc((void **)&s.Epre, n * sizeof(double)) && alloc((void **)&s.W, 2 * (nf + 1) * n * sizeof(double));
  }
  g_slot.s    = s;
  g_slot.live = true;
  if (!ok) {
    cudaGetLastError();
    free_slot(g_slot);
    return fail(CGB_ERR_NOMEM, "scratch allocation failed");
  }
  g_slot.nx = nx, g_slot.ny = ny, g_slot.nz = nz, g_slot.nf = nf, g_slot.mhd = mhd, g_slot.dev = dev;
  return CGB_OK;
}

int check_scheme(const cgb_scheme &s)
{
  if (s.reconstruction < CGB_PCM || s.reconstruction > CGB_PPMP) return fail(CGB_ERR_ARGS, "bad reconstruction");
  if (s.riemann_solver < CGB_HLLC || s.riemann_solver > CGB_EXACT) return fail(CGB_ERR_ARGS, "bad riemann solver");
  if (s.n_scalars < 0 || s.n_scalars > cgb::NS_MAX) return fail(CGB_ERR_ARGS, "n_scalars must be 0..2");
  if (!(s.gamma > 1.0)) return fail(CGB_ERR_ARGS, "gamma must exceed 1");
  if (s.mhd && s.riemann_solver != CGB_HLLD) return fail(CGB_ERR_ARGS, "MHD needs the HLLD solver");
  if (!s.mhd && s.riemann_solver == CGB_HLLD) return fail(CGB_ERR_ARGS, "HLLD needs MHD");
  if (s.mhd && s.dual_energy)
    return fail(CGB_ERR_UNSUPPORTED, "MHD with dual energy is not supported (the reference indexes past its flux arrays)");
  if (s.precision < CGB_FP64 || s.precision > CGB_FP64_FAST) return fail(CGB_ERR_ARGS, "bad precision");
  return CGB_OK;
}

// ghost layers the reconstruction's stencil needs (the reference's n_ghost, grid3D.cpp:53-76)
int ghosts_needed(const cgb_scheme &s)
{
  switch (s.reconstruction) {
    case CGB_PPMC:
    case CGB_PPMP: return 4;
    case CGB_PLMC:
    case CGB_PLMP: return 3;
    default: return 2;
  }
}

int expected_fields(const cgb_scheme &s) { return 5 + s.n_scalars + (s.mhd ? 3 : 0) + (s.dual_energy ? 1 : 0); }

int make_box(cgb::Box &b, int nx, int ny, int nz, int ng, int nf, double dx, double dy, double dz,
             double density_floor, const cgb_scheme &s)
{
  if (nx < 1 || ny < 1 || nz < 1 || ng < 1) return fail(CGB_ERR_ARGS, "bad grid size");
  if (nf != expected_fields(s)) return fail(CGB_ERR_ARGS, "n_fields does not match the scheme");
  if (!(dx > 0) || !(dy > 0) || !(dz > 0)) return fail(CGB_ERR_ARGS, "cell sizes must be positive");
  b.nx = nx, b.ny = ny, b.nz = nz, b.ng = ng, b.nf = nf, b.ns = s.n_scalars;
  b.de = s.dual_energy ? 1 : 0;
  b.mhd = s.mhd ? 1 : 0;
  b.floor_on = s.density_floor ? 1 : 0;
  b.n = (long long)nx * ny * nz;
  b.gamma = s.gamma;
  b.dx = dx, b.dy = dy, b.dz = dz;
  b.density_floor = density_floor;
  return CGB_OK;
}
}  // namespace

// Static scratch of cgb_vl_algorithm_3d_static: a file-scope array in the module's static device
// memory, which the CUDA driver provides when it loads the module; no call allocates it.  A box of n
// padded cells and f fields needs (f + 2) 8 n bytes in exact FP64 and (2 f + 4) 8 n in the fast
// forms (each array rounded to 256 bytes) plus 512: with 6 fields, 24 MiB holds fewer than
// 393,216 padded cells (73^3) in FP64 and fewer than 196,608 (58^3) in fast FP64 / mixed.
constexpr size_t kStaticScratchBytes = size_t(24) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

namespace
{
constexpr int kMaxDevices = 64;
void *g_static_pool[kMaxDevices] = {};  // device address of g_static_scratch, per device ordinal

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// One-word results of the device reductions (0: CFL max, 1: max |div B|), one per device.
unsigned long long *g_word[kMaxDevices][2] = {};

int device_word(int which, unsigned long long **word)
{
  int dev       = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(CGB_ERR_ARGS, "device ordinal beyond the result-word table");
  if (!g_word[dev][which] && cgb::dev_malloc((void **)&g_word[dev][which], sizeof(unsigned long long)) != cudaSuccess) {
    g_word[dev][which] = nullptr;
    cudaGetLastError();
    return fail(CGB_ERR_NOMEM, "reduction result word");
  }
  *word = g_word[dev][which];
  return CGB_OK;
}

// Bytes of static scratch one step of box b needs in the given arithmetic, and (base != null)
// the Scratch pointers laid out from base, each array on a 256-byte boundary.
size_t static_layout(const cgb::Box &b, int precision, unsigned char *base, cgb::Scratch *out)
{
  size_t const n = (size_t)b.n, nf = (size_t)b.nf;
  size_t off = 0;
  auto take  = [&](size_t bytes) -> void * {
    size_t const o = off;
    off += align256(bytes);
    return base ? base + o : nullptr;
  };
  cgb::Scratch sc{};
  sc.status = (int *)take(sizeof(int));
  sc.dti    = (unsigned long long *)take(sizeof(unsigned long long));
  sc.GEp    = (double *)take(n * sizeof(double));
  sc.Epre   = (double *)take(n * sizeof(double));
  if (precision == CGB_FP64)
    sc.Uh = (double *)take(nf * n * sizeof(double));  // U at the half step
  else
    sc.W = take(2 * (nf + 1) * n * sizeof(double));  // primitives of U^n and of U^(n+1/2)
  if (out) *out = sc;
  return off;
}

// Device address of the static pool on the current device, looked up once per device.
int static_pool(void **pool)
{
  int dev       = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(CGB_ERR_ARGS, "device ordinal beyond the static pool table");
  if (!g_static_pool[dev]) {
    void *p = nullptr;
    e       = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
    g_static_pool[dev] = p;
  }
  *pool = g_static_pool[dev];
  return CGB_OK;
}
}  // namespace

extern "C" {

const char *cgb_last_error(void) { return g_err.c_str(); }
const char *cgb_version(void) { return "cholla_gb300 0.1 (sm_103a)"; }

int cgb_set_scheme(const cgb_scheme *scheme)
{
  if (!scheme) return fail(CGB_ERR_ARGS, "null scheme");
  int const rc = check_scheme(*scheme);
  if (rc != CGB_OK) return rc;
  std::lock_guard<std::mutex> lk(g_mu);
  g_scheme = *scheme;
  return CGB_OK;
}

int cgb_get_scheme(cgb_scheme *scheme)
{
  if (!scheme) return fail(CGB_ERR_ARGS, "null scheme");
  std::lock_guard<std::mutex> lk(g_mu);
  *scheme = g_scheme;
  return CGB_OK;
}

int cgb_set_stream(void *stream)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_stream = (cudaStream_t)stream;
  return CGB_OK;
}

int cgb_vl_algorithm_3d(double *d_conserved, double *d_grav_potential, int nx, int ny, int nz, int x_off, int y_off,
                        int z_off, int n_ghost, double dx, double dy, double dz, double xbound, double ybound,
                        double zbound, double dt, int n_fields, int custom_grav, double density_floor,
                        double *host_grav_potential)
{
  (void)x_off, (void)y_off, (void)z_off, (void)xbound, (void)ybound, (void)zbound;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved) return fail(CGB_ERR_ARGS, "null d_conserved");
  if (d_grav_potential || host_grav_potential || custom_grav)
    return fail(CGB_ERR_UNSUPPORTED, "gravity source terms are not part of this library");
  if (ny < 2 * n_ghost + 1 || nz < 2 * n_ghost + 1 || nx < 2 * n_ghost + 1)
    return fail(CGB_ERR_ARGS, "3D step needs at least one real cell per dimension");
  cgb::Box b;
  int rc = make_box(b, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, density_floor, g_scheme);
  if (rc != CGB_OK) return rc;
  int const H = ghosts_needed(g_scheme) + (g_scheme.mhd ? 1 : 0);
  if (n_ghost < H) return fail(CGB_ERR_ARGS, "n_ghost too small for the reconstruction");
  if (g_scheme.mhd && g_scheme.precision == CGB_MIXED)
    return fail(CGB_ERR_UNSUPPORTED, "the MHD step is built in exact and fast FP64 only");
  rc = ensure_slot(nx, ny, nz, n_fields, g_scheme.mhd);
  if (rc != CGB_OK) return rc;
  if (g_scheme.mhd) {
    cudaError_t e = cgb::mhd_step(b, g_scheme.reconstruction, g_scheme.precision, d_conserved, g_slot.s.mhd, dt, nullptr,
                                  g_stream);
    if (e != cudaSuccess) return cuda_fail(e, "vl_algorithm_3d (MHD)");
    return CGB_OK;
  }
  cudaError_t e = cgb::hydro_step(b, g_scheme.reconstruction, g_scheme.riemann_solver, g_scheme.precision,
                                  d_conserved, g_slot.s, dt, nullptr, 0.0, 0, 0, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "vl_algorithm_3d");
  return CGB_OK;
}

int cgb_vl_algorithm_3d_static(double *d_conserved, double *d_grav_potential, int nx, int ny, int nz, int x_off,
                               int y_off, int z_off, int n_ghost, double dx, double dy, double dz, double xbound,
                               double ybound, double zbound, double dt, int n_fields, int custom_grav,
                               double density_floor, double *host_grav_potential)
{
  (void)x_off, (void)y_off, (void)z_off, (void)xbound, (void)ybound, (void)zbound;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved) return fail(CGB_ERR_ARGS, "null d_conserved");
  if (d_grav_potential || host_grav_potential || custom_grav)
    return fail(CGB_ERR_UNSUPPORTED, "gravity source terms are not part of this library");
  if (ny < 2 * n_ghost + 1 || nz < 2 * n_ghost + 1 || nx < 2 * n_ghost + 1)
    return fail(CGB_ERR_ARGS, "3D step needs at least one real cell per dimension");
  cgb::Box b;
  int rc = make_box(b, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, density_floor, g_scheme);
  if (rc != CGB_OK) return rc;
  int const H = ghosts_needed(g_scheme);
  if (n_ghost < H) return fail(CGB_ERR_ARGS, "n_ghost too small for the reconstruction");
  if (g_scheme.mhd) return fail(CGB_ERR_UNSUPPORTED, "the static-pool step is hydro only");
  size_t const need = static_layout(b, g_scheme.precision, nullptr, nullptr);
  if (need > kStaticScratchBytes)
    return fail(CGB_ERR_ARGS, "box needs " + std::to_string(need) + " bytes of scratch but the static pool of "
                              "cgb_vl_algorithm_3d_static holds " + std::to_string(kStaticScratchBytes) +
                              "; use cgb_vl_algorithm_3d for this box");
  void *pool = nullptr;
  rc         = static_pool(&pool);
  if (rc != CGB_OK) return rc;
  cgb::Scratch sc;
  static_layout(b, g_scheme.precision, (unsigned char *)pool, &sc);
  // the status word collects bad-cell flags with atomicOr, so it must start at zero; every
  // other array is written before it is read within the step
  cudaError_t e = cudaMemsetAsync(sc.status, 0, sizeof(int), g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "clear static status word");
  e = cgb::hydro_step(b, g_scheme.reconstruction, g_scheme.riemann_solver, g_scheme.precision, d_conserved, sc, dt,
                      nullptr, 0.0, 0, 0, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "vl_algorithm_3d_static");
  return CGB_OK;
}

int cgb_vl_algorithm_1d(double *d_conserved, int nx, int x_off, int n_ghost, double dx, double xbound, double dt,
                        int n_fields, int custom_grav)
{
  (void)x_off, (void)xbound;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved) return fail(CGB_ERR_ARGS, "null d_conserved");
  if (custom_grav) return fail(CGB_ERR_UNSUPPORTED, "gravity source terms are not part of this library");
  if (g_scheme.mhd) return fail(CGB_ERR_UNSUPPORTED, "the 1D integrator is hydro only");
  if (g_scheme.riemann_solver == CGB_HLL)
    return fail(CGB_ERR_UNSUPPORTED, "the reference's 1D integrator has no HLL branch (VL_1D_cuda.cu)");
  if (nx < 2 * n_ghost + 1) return fail(CGB_ERR_ARGS, "1D step needs at least one real cell");
  cgb::Box b;
  int rc = make_box(b, nx, 1, 1, n_ghost, n_fields, dx, dx, dx, 0.0, g_scheme);
  if (rc != CGB_OK) return rc;
  b.floor_on = 0;  // the 1D updates apply no density floor (hydro_cuda.cu:20-82, VL_1D_cuda.cu:158-215)
  rc = ensure_slot(nx, 1, 1, n_fields, 0);
  if (rc != CGB_OK) return rc;
  cudaError_t e = cgb::hydro_step(b, g_scheme.reconstruction, g_scheme.riemann_solver, g_scheme.precision,
                                  d_conserved, g_slot.s, dt, nullptr, 0.0, 0, 0, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "vl_algorithm_1d");
  return CGB_OK;
}

int cgb_vl_algorithm_2d(double *d_conserved, int nx, int ny, int x_off, int y_off, int n_ghost, double dx, double dy,
                        double xbound, double ybound, double dt, int n_fields, int custom_grav)
{
  (void)x_off, (void)y_off, (void)xbound, (void)ybound;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved) return fail(CGB_ERR_ARGS, "null d_conserved");
  if (custom_grav) return fail(CGB_ERR_UNSUPPORTED, "gravity source terms are not part of this library");
  if (g_scheme.mhd) return fail(CGB_ERR_UNSUPPORTED, "the 2D integrator is hydro only");
  if (g_scheme.riemann_solver == CGB_HLL)
    return fail(CGB_ERR_UNSUPPORTED, "the reference's 2D integrator has no HLL branch (VL_2D_cuda.cu)");
  if (g_scheme.precision != CGB_FP64)
    return fail(CGB_ERR_UNSUPPORTED, "the 2D step is built in the exact FP64 form (CGB_FP64) only");
  if (nx < 2 * n_ghost + 1 || ny < 2 * n_ghost + 1) return fail(CGB_ERR_ARGS, "2D step needs real cells in x and y");
  cgb::Box b;
  int rc = make_box(b, nx, ny, 1, n_ghost, n_fields, dx, dy, dx, 0.0, g_scheme);
  if (rc != CGB_OK) return rc;
  b.floor_on = 0;  // the 2D updates apply no density floor (VL_2D_cuda.cu:176-258, hydro_cuda.cu:87-170)
  if (n_ghost < ghosts_needed(g_scheme)) return fail(CGB_ERR_ARGS, "n_ghost too small for the reconstruction");
  rc = ensure_slot(nx, ny, 1, n_fields, 0);
  if (rc != CGB_OK) return rc;
  cudaError_t e = cgb::hydro_step(b, g_scheme.reconstruction, g_scheme.riemann_solver, CGB_FP64, d_conserved,
                                  g_slot.s, dt, nullptr, 0.0, 0, 0, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "vl_algorithm_2d");
  return CGB_OK;
}

int cgb_free_memory_vl_3d(void)
{
  std::lock_guard<std::mutex> lk(g_mu);
  free_slot(g_slot);
  return CGB_OK;
}

int cgb_calc_dt_gpu(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx,
                    double dy, double dz, double gamma, double *max_dti)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved || !max_dti) return fail(CGB_ERR_ARGS, "null pointer");
  (void)n_fields;  // as in the reference (the caller passes n_cells here, grid3D.cpp:119)
  cgb_scheme s = g_scheme;
  s.gamma      = gamma;
  cgb::Box b;
  b.nx = nx, b.ny = ny, b.nz = nz, b.ng = n_ghost, b.nf = expected_fields(s), b.ns = s.n_scalars;
  b.de = s.dual_energy, b.mhd = s.mhd, b.floor_on = 0, b.n = (long long)nx * ny * nz, b.gamma = gamma;
  b.dx = dx, b.dy = dy, b.dz = dz, b.density_floor = 0;
  if (b.mhd && !(ny > 1 && nz > 1)) return fail(CGB_ERR_ARGS, "MHD boxes are 3D");
  if (!(nx > 1 && ((ny == 1 && nz == 1) || ny > 1))) return fail(CGB_ERR_ARGS, "1D, 2D (nz = 1) or 3D boxes only");
  if (b.mhd && nz == 1) return fail(CGB_ERR_ARGS, "MHD boxes are 3D");
  unsigned long long *d_dti = nullptr;
  int const rw               = device_word(0, &d_dti);
  if (rw != CGB_OK) return rw;
  cudaError_t e = b.mhd ? cgb::mhd_calc_dt(b, d_conserved, d_dti, g_stream)
                        : cgb::hydro_calc_dt(b, d_conserved, d_dti, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "calc_dt");
  unsigned long long bits = 0;
  int const rr            = read_word(d_dti, &bits, "calc_dt readback");
  if (rr != CGB_OK) return rr;
  double v;
  std::memcpy(&v, &bits, sizeof(v));
  *max_dti = bits == 0 ? 0.0 : v;
  return CGB_OK;
}

int cgb_apply_temperature_floor(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                double U_floor)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved) return fail(CGB_ERR_ARGS, "null d_conserved");
  cgb::Box b;
  int rc = make_box(b, nx, ny, nz, n_ghost, n_fields, 1.0, 1.0, 1.0, 0.0, g_scheme);
  if (rc != CGB_OK) return rc;
  cudaError_t e = cgb::hydro_temperature_floor(b, d_conserved, U_floor, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "temperature floor");
  return CGB_OK;
}

int cgb_set_boundaries(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, const int flags[6])
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved || !flags) return fail(CGB_ERR_ARGS, "null pointer");
  for (int i = 0; i < 6; i++)
    if (flags[i] < 0 || flags[i] > 5) return fail(CGB_ERR_ARGS, "boundary flags must be 0..5");
  cgb::Box b;
  b.nx = nx, b.ny = ny, b.nz = nz, b.ng = n_ghost, b.nf = n_fields, b.ns = g_scheme.n_scalars;
  b.de = g_scheme.dual_energy, b.mhd = g_scheme.mhd, b.floor_on = 0, b.n = (long long)nx * ny * nz;
  b.gamma = g_scheme.gamma, b.dx = b.dy = b.dz = 1.0, b.density_floor = 0;
  if (nx < 1 || ny < 1 || nz < 1 || n_ghost < 1 || n_fields < 5) return fail(CGB_ERR_ARGS, "bad grid");
  cudaError_t e = cgb::set_boundaries(b, d_conserved, flags, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "set_boundaries");
  return CGB_OK;
}

int cgb_max_magnetic_divergence(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                double dx, double dy, double dz, double *max_divb)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!d_conserved || !max_divb) return fail(CGB_ERR_ARGS, "null pointer");
  if (!g_scheme.mhd) return fail(CGB_ERR_ARGS, "the scheme has no magnetic field");
  cgb::Box b;
  int const rc = make_box(b, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, 0.0, g_scheme);
  if (rc != CGB_OK) return rc;
  if (ny < 2 || nz < 2) return fail(CGB_ERR_ARGS, "MHD boxes are 3D");
  unsigned long long *d_div = nullptr;
  int const rw               = device_word(1, &d_div);
  if (rw != CGB_OK) return rw;
  cudaError_t e = cgb::mhd_max_divb(b, d_conserved, d_div, g_stream);
  if (e != cudaSuccess) return cuda_fail(e, "max_magnetic_divergence");
  unsigned long long bits = 0;
  int const rr            = read_word(d_div, &bits, "max_magnetic_divergence readback");
  if (rr != CGB_OK) return rr;
  std::memcpy(max_divb, &bits, sizeof(double));
  return CGB_OK;
}

int cgb_check_magnetic_divergence(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                  double dx, double dy, double dz, double *max_divb)
{
  double v  = 0.0;
  int const rc = cgb_max_magnetic_divergence(d_conserved, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, &v);
  if (max_divb) *max_divb = v;
  if (rc != CGB_OK) return rc;
  // magnetic_divergence.cu:105-116: the limit, and a negative (or NaN) maximum, are fatal there
  if (!(v >= 0.0) || v > CGB_MAX_DIVB) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "magnetic divergence %.4e exceeds the limit %.1e (or is not a number)", v,
                  CGB_MAX_DIVB);
    return fail(CGB_ERR_NONFINITE, buf);
  }
  return CGB_OK;
}

int cgb_check_status(int *flags)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (flags) *flags = 0;
  if (!g_slot.live || !g_slot.s.status) return CGB_OK;
  int cur = -1;
  bool const other = cudaGetDevice(&cur) == cudaSuccess && g_slot.dev != cur;
  if (other) cudaSetDevice(g_slot.dev);
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, g_slot.s.status, sizeof(int), cudaMemcpyDeviceToHost, g_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(g_slot.s.status, 0, sizeof(int), g_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_stream);
  if (other) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "check_status");
  if (flags) *flags = h;
  if (h & CGB_STATUS_TIMEOUT)
    return fail(CGB_ERR_TIMEOUT, "a bounded device wait for a TMA copy ran out; the step left a tile undone");
  if (h & CGB_STATUS_NONFINITE)
    return fail(CGB_ERR_NONFINITE, "a step left a real cell with non-finite density or energy, or density <= 0 "
                                   "after the negative-density repair");
  return CGB_OK;
}

}  // extern "C"
