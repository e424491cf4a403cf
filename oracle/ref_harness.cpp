// ref_harness.cpp -- runs the reference's own CUDA kernels (cubins built from the cholla
// source tree by oracle/build_ref.sh) in the order of VL_Algorithm_3D_CUDA
// (src/integrators/VL_3D_cuda.cu:38-360), VL_Algorithm_1D_CUDA (VL_1D_cuda.cu:30-146),
// Calc_dt_GPU (hydro_cuda.cu:562-597), Apply_Temperature_Floor and the ghost-cell fill
// (cuda_boundaries.cu:71-160, boundary_conditions.cpp:165-500).
//
// TEST INFRASTRUCTURE ONLY: the parity baseline ("the reference's own build on the same
// GPU") and its timing.  It uses the CUDA driver API on the primary context, so device
// pointers from torch can be passed straight in.  Kernel names are the Itanium-mangled
// names of the reference's kernels.
#include <cuda.h>
#include <dirent.h>

#include <cfloat>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace
{
std::string g_err;
CUcontext g_ctx = nullptr;
std::vector<CUmodule> g_mods;
std::map<std::string, CUfunction> g_fn;
bool g_de = false, g_mhd = false;
int g_recon = 2;   // 1 PLMC, 2 PPMC, 3 PLMP, 4 PPMP
int g_solver = 0;  // 0 HLLC, 1 ROE, 2 HLLD, 3 HLL, 4 exact
struct Scratch {
  size_t n = 0;
  int nf = 0;
  CUdeviceptr Uh = 0, QLx = 0, QRx = 0, QLy = 0, QRy = 0, QLz = 0, QRz = 0, Fx = 0, Fy = 0, Fz = 0, emf = 0, dti = 0;
} g_s;
CUstream g_stream = nullptr;
// the reference's default build synchronises the device after every kernel (GPU_Error_Check ->
// cudaDeviceSynchronize, src/utils/gpu.hpp:139-155); -DDISABLE_GPU_ERROR_CHECKING removes it
bool g_sync_each = false;

int err(const std::string &m)
{
  g_err = m;
  return 1;
}
int cu(CUresult r, const char *what)
{
  if (r == CUDA_SUCCESS) return 0;
  const char *s = nullptr;
  cuGetErrorString(r, &s);
  return err(std::string(what) + ": " + (s ? s : "?"));
}

CUfunction fn(const char *name)
{
  auto it = g_fn.find(name);
  if (it != g_fn.end()) return it->second;
  for (CUmodule m : g_mods) {
    CUfunction f;
    if (cuModuleGetFunction(&f, m, name) == CUDA_SUCCESS) {
      g_fn[name] = f;
      return f;
    }
  }
  return nullptr;
}

template <typename... A>
int launch(const char *name, size_t nthreads, A... args)
{
  CUfunction f = fn(name);
  if (!f) return err(std::string("kernel not found in the reference cubins: ") + name);
  void *p[] = {(void *)&args...};
  unsigned const tpb  = 256;
  unsigned const grid = (unsigned)((nthreads + tpb - 1) / tpb);
  if (cu(cuLaunchKernel(f, grid, 1, 1, tpb, 1, 1, 0, g_stream, p, nullptr), name)) return 1;
  return g_sync_each ? cu(cuCtxSynchronize(), name) : 0;
}

void free_scratch()
{
  CUdeviceptr *ps[] = {&g_s.Uh, &g_s.QLx, &g_s.QRx, &g_s.QLy, &g_s.QRy, &g_s.QLz, &g_s.QRz,
                       &g_s.Fx, &g_s.Fy, &g_s.Fz, &g_s.emf, &g_s.dti};
  for (auto p : ps)
    if (*p) cuMemFree(*p), *p = 0;
  g_s.n = 0;
}

int ensure_scratch(size_t n, int nf)
{
  if (g_s.n == n && g_s.nf == nf) return 0;
  free_scratch();
  size_t const nif = g_mhd ? nf - 1 : nf;
  auto al = [&](CUdeviceptr *p, size_t bytes) {
    if (cuMemAlloc(p, bytes) != CUDA_SUCCESS) return false;
    return cuMemsetD8(*p, 0, bytes) == CUDA_SUCCESS;  // initGpuMemory (cuda_utilities.h:80)
  };
  bool ok = al(&g_s.Uh, n * nf * 8) && al(&g_s.QLx, n * nif * 8) && al(&g_s.QRx, n * nif * 8) &&
            al(&g_s.QLy, n * nif * 8) && al(&g_s.QRy, n * nif * 8) && al(&g_s.QLz, n * nif * 8) &&
            al(&g_s.QRz, n * nif * 8) && al(&g_s.Fx, n * nif * 8) && al(&g_s.Fy, n * nif * 8) &&
            al(&g_s.Fz, n * nif * 8) && al(&g_s.dti, 8) && (!g_mhd || al(&g_s.emf, 3 * n * 8));
  if (!ok) {
    free_scratch();
    return err("reference scratch allocation failed");
  }
  // the zeroing above runs on the legacy stream, which a non-blocking caller stream does not wait
  // for: finish it before any kernel of that stream touches the scratch
  if (cu(cuCtxSynchronize(), "scratch zeroing")) return 1;
  g_s.n  = n;
  g_s.nf = nf;
  return 0;
}

const char *K_PCM3    = "_Z21PCM_Reconstruction_3DPdS_S_S_S_S_S_iiiidi";
const char *K_PCM1    = "_Z21PCM_Reconstruction_1DPdS_S_iidi";
const char *K_HLLC    = "_Z26Calculate_HLLC_Fluxes_CUDAPdS_S_iiiidii";
const char *K_ROE     = "_Z25Calculate_Roe_Fluxes_CUDAPdS_S_iiiidii";
const char *K_HLLD    = "_ZN3mhd26Calculate_HLLD_Fluxes_CUDAEPKdS1_S1_Pdidii";
const char *K_HLL     = "_Z25Calculate_HLL_Fluxes_CUDAPdS_S_iiiidii";
const char *K_EXACT   = "_Z27Calculate_Exact_Fluxes_CUDAPdS_S_iiiidii";
const char *K_CT      = "_ZN3mhd28Calculate_CT_Electric_FieldsEPKdS1_S1_S1_Pdiiii";
const char *K_BUPD    = "_ZN3mhd24Update_Magnetic_Field_3DEPdS0_S0_iiiidddd";
const char *K_DIVB    = "_ZN3mhd27calculateMagneticDivergenceEPKdPddddiiii";
const char *K_HALF3   = "_Z34Update_Conserved_Variables_3D_halfPdS_S_S_S_iiiidddddid";
const char *K_HALF1   = "_Z34Update_Conserved_Variables_1D_halfPdS_S_iidddi";
const char *K_PPMC    = "_Z7PPMC_VLPdS_S_iiidi";
const char *K_PLMC    = "_Z9PLMC_cudaPdS_S_iiidddii";
const char *K_PLMP    = "_Z9PLMP_cudaPdS_S_iiiidddii";
const char *K_PPMP    = "_Z9PPMP_cudaPdS_S_iiiidddii";
const char *K_DEP3    = "_Z42Partial_Update_Advected_Internal_Energy_3DPdS_S_S_S_S_S_iiiidddddi";
const char *K_DEP1    = "_Z42Partial_Update_Advected_Internal_Energy_1DPdS_S_iidddi";
const char *K_UPD3    = "_Z29Update_Conserved_Variables_3DPdS_S_S_S_S_S_S_S_S_iiiiiiiddddddddiidS_";
const char *K_UPD1    = "_Z29Update_Conserved_Variables_1DPdS_iiiddddii";
const char *K_SEL3    = "_Z25Select_Internal_Energy_3DPdiiiii";
const char *K_SEL1    = "_Z25Select_Internal_Energy_1DPdiii";
const char *K_SYNC3   = "_Z16Sync_Energies_3DPdiiiidi";
const char *K_SYNC1   = "_Z16Sync_Energies_1DPdiidi";
const char *K_DT3     = "_Z10Calc_dt_3DPdS_diiiiiddd";
const char *K_DT1     = "_Z10Calc_dt_1DPdS_diid";
const char *K_TFLOOR  = "_Z24Temperature_Floor_KernelPdiiiiid";
const char *K_GHOST   = "_Z19SetGhostCellsKernelPdiiiiiiiiiiiiiiiiiii";

int riemann(CUdeviceptr QL, CUdeviceptr QR, CUdeviceptr F, CUdeviceptr Bface, int nx, int ny, int nz, int ng,
            double gamma, int dir, int nf)
{
  size_t const n = (size_t)nx * ny * nz;
  if (g_solver == 2) return launch(K_HLLD, n, QL, QR, Bface, F, (int)n, gamma, dir, nf);
  const char *k = g_solver == 1 ? K_ROE : g_solver == 3 ? K_HLL : g_solver == 4 ? K_EXACT : K_HLLC;
  return launch(k, n, QL, QR, F, nx, ny, nz, ng, gamma, dir, nf);
}
}  // namespace

extern "C" {

const char *refh_error(void) { return g_err.c_str(); }

// Load every cubin of one variant directory (oracle/_ref/<variant>/); the variant name
// gives the compile-time options (e.g. hydro_ppmc_hllc_de, mhd_plmc_hlld).
int refh_init(const char *variant_dir, const char *variant)
{
  if (cu(cuInit(0), "cuInit")) return 1;
  CUdevice d;
  if (cu(cuDeviceGet(&d, 0), "cuDeviceGet")) return 1;
  if (cu(cuDevicePrimaryCtxRetain(&g_ctx, d), "primary context")) return 1;
  if (cu(cuCtxSetCurrent(g_ctx), "set context")) return 1;
  for (CUmodule m : g_mods) cuModuleUnload(m);
  g_mods.clear();
  g_fn.clear();
  free_scratch();
  std::string v(variant);
  g_de     = v.find("_de") != std::string::npos;
  g_mhd    = v.rfind("mhd", 0) == 0;
  auto has = [&v](const char *t) { return v.find(t) != std::string::npos; };
  g_recon  = has("plmc") ? 1 : has("plmp") ? 3 : has("ppmp") ? 4 : 2;
  // "hllc" and "hlld" contain "hll": test them first
  g_solver = has("hlld") ? 2 : has("roe") ? 1 : has("exact") ? 4 : (has("_hll") && !has("_hllc")) ? 3 : 0;
  DIR *dir = opendir(variant_dir);
  if (!dir) return err(std::string("no reference cubins at ") + variant_dir);
  while (dirent *e = readdir(dir)) {
    std::string name = e->d_name;
    if (name.size() < 6 || name.substr(name.size() - 6) != ".cubin") continue;
    CUmodule m;
    if (cu(cuModuleLoad(&m, (std::string(variant_dir) + "/" + name).c_str()), name.c_str())) {
      closedir(dir);
      return 1;
    }
    g_mods.push_back(m);
  }
  closedir(dir);
  return g_mods.empty() ? err("no cubins loaded") : 0;
}

int refh_set_stream(void *s)
{
  g_stream = (CUstream)s;
  return 0;
}

// VL_Algorithm_3D_CUDA with its DENSITY_FLOOR / DE / MHD branches, gravity off.
int refh_vl_step_3d(unsigned long long U_, int nx, int ny, int nz, int ng, double dx, double dy, double dz, double dt,
                    int nf, double gamma, double density_floor)
{
  CUdeviceptr U  = (CUdeviceptr)U_;
  size_t const n = (size_t)nx * ny * nz;
  if (ensure_scratch(n, nf)) return 1;
  Scratch &s = g_s;
  int const fB = nf - 3 - (g_de ? 1 : 0);
  auto face    = [&](CUdeviceptr base, int k) { return base + (CUdeviceptr)((size_t)(fB + k) * n * 8); };
  int const in = (int)n;
  if (launch(K_PCM3, n, U, s.QLx, s.QRx, s.QLy, s.QRy, s.QLz, s.QRz, nx, ny, nz, ng, gamma, nf)) return 1;
  if (riemann(s.QLx, s.QRx, s.Fx, g_mhd ? face(U, 0) : 0, nx, ny, nz, ng, gamma, 0, nf)) return 1;
  if (riemann(s.QLy, s.QRy, s.Fy, g_mhd ? face(U, 1) : 0, nx, ny, nz, ng, gamma, 1, nf)) return 1;
  if (riemann(s.QLz, s.QRz, s.Fz, g_mhd ? face(U, 2) : 0, nx, ny, nz, ng, gamma, 2, nf)) return 1;
  if (g_mhd && launch(K_CT, n, s.Fx, s.Fy, s.Fz, U, s.emf, nx, ny, nz, in)) return 1;
  if (launch(K_HALF3, n, U, s.Uh, s.Fx, s.Fy, s.Fz, nx, ny, nz, ng, dx, dy, dz, 0.5 * dt, gamma, nf, density_floor))
    return 1;
  if (g_mhd && launch(K_BUPD, n, U, s.Uh, s.emf, nx, ny, nz, in, 0.5 * dt, dx, dy, dz)) return 1;
  CUdeviceptr QL[3] = {s.QLx, s.QLy, s.QLz}, QR[3] = {s.QRx, s.QRy, s.QRz}, F[3] = {s.Fx, s.Fy, s.Fz};
  double const dd[3] = {dx, dy, dz};
  for (int d = 0; d < 3; d++) {
    if (g_recon == 2) {
      if (launch(K_PPMC, n, s.Uh, QL[d], QR[d], nx, ny, nz, gamma, d)) return 1;
    } else if (g_recon >= 3) {
      if (launch(g_recon == 3 ? K_PLMP : K_PPMP, n, s.Uh, QL[d], QR[d], nx, ny, nz, ng, dd[d], dt, gamma, d, nf))
        return 1;
    } else {
      if (launch(K_PLMC, n, s.Uh, QL[d], QR[d], nx, ny, nz, dd[d], dt, gamma, d, nf)) return 1;
    }
  }
  for (int d = 0; d < 3; d++)
    if (riemann(QL[d], QR[d], F[d], g_mhd ? face(s.Uh, d) : 0, nx, ny, nz, ng, gamma, d, nf)) return 1;
  if (g_de && launch(K_DEP3, n, U, s.QLx, s.QRx, s.QLy, s.QRy, s.QLz, s.QRz, nx, ny, nz, ng, dx, dy, dz, dt, gamma, nf))
    return 1;
  if (g_mhd && launch(K_CT, n, s.Fx, s.Fy, s.Fz, s.Uh, s.emf, nx, ny, nz, in)) return 1;
  CUdeviceptr nullp = 0;
  int const zero = 0;
  double const zd = 0.0;
  if (launch(K_UPD3, n, U, s.QLx, s.QRx, s.QLy, s.QRy, s.QLz, s.QRz, s.Fx, s.Fy, s.Fz, nx, ny, nz, zero, zero, zero, ng,
             dx, dy, dz, zd, zd, zd, dt, gamma, nf, zero, density_floor, nullp))
    return 1;
  if (g_mhd && launch(K_BUPD, n, U, U, s.emf, nx, ny, nz, in, dt, dx, dy, dz)) return 1;
  if (g_de) {
    if (launch(K_SEL3, n, U, nx, ny, nz, ng, nf)) return 1;
    if (launch(K_SYNC3, n, U, nx, ny, nz, ng, gamma, nf)) return 1;
  }
  return 0;
}

// VL_Algorithm_1D_CUDA (hydro).
int refh_vl_step_1d(unsigned long long U_, int nx, int ng, double dx, double dt, int nf, double gamma)
{
  CUdeviceptr U  = (CUdeviceptr)U_;
  size_t const n = (size_t)nx;
  if (ensure_scratch(n, nf)) return 1;
  Scratch &s = g_s;
  int const one = 1;
  if (launch(K_PCM1, n, U, s.QLx, s.QRx, nx, ng, gamma, nf)) return 1;
  if (riemann(s.QLx, s.QRx, s.Fx, 0, nx, 1, 1, ng, gamma, 0, nf)) return 1;
  if (launch(K_HALF1, n, U, s.Uh, s.Fx, nx, ng, dx, 0.5 * dt, gamma, nf)) return 1;
  if (g_recon == 2) {
    if (launch(K_PPMC, n, s.Uh, s.QLx, s.QRx, nx, one, one, gamma, 0)) return 1;
  } else if (g_recon >= 3) {
    if (launch(g_recon == 3 ? K_PLMP : K_PPMP, n, s.Uh, s.QLx, s.QRx, nx, one, one, ng, dx, dt, gamma, 0, nf))
      return 1;
  } else {
    if (launch(K_PLMC, n, s.Uh, s.QLx, s.QRx, nx, one, one, dx, dt, gamma, 0, nf)) return 1;
  }
  if (riemann(s.QLx, s.QRx, s.Fx, 0, nx, 1, 1, ng, gamma, 0, nf)) return 1;
  if (g_de && launch(K_DEP1, n, U, s.QLx, s.QRx, nx, ng, dx, dt, gamma, nf)) return 1;
  int const zero = 0;
  double const zd = 0.0;
  if (launch(K_UPD1, n, U, s.Fx, nx, zero, ng, dx, zd, dt, gamma, nf, zero)) return 1;
  if (g_de) {
    if (launch(K_SEL1, n, U, nx, ng, nf)) return 1;
    if (launch(K_SYNC1, n, U, nx, ng, gamma, nf)) return 1;
  }
  return 0;
}

// Calc_dt_GPU: returns the maximum inverse crossing time (synchronises).
int refh_calc_dt(unsigned long long U_, int nx, int ny, int nz, int ng, int nf, double dx, double dy, double dz,
                 double gamma, double *out)
{
  CUdeviceptr U = (CUdeviceptr)U_;
  if (ensure_scratch((size_t)nx * ny * nz, nf)) return 1;
  double const lowest = -DBL_MAX;
  if (cu(cuMemcpyHtoDAsync(g_s.dti, &lowest, 8, g_stream), "dti init")) return 1;
  if (cu(cuStreamSynchronize(g_stream), "sync")) return 1;
  size_t const n = (size_t)nx * ny * nz;
  if (ny == 1 && nz == 1) {
    if (launch(K_DT1, n, U, g_s.dti, gamma, ng, nx, dx)) return 1;
  } else {
    if (launch(K_DT3, n, U, g_s.dti, gamma, ng, nf, nx, ny, nz, dx, dy, dz)) return 1;
  }
  if (cu(cuStreamSynchronize(g_stream), "sync")) return 1;
  return cu(cuMemcpyDtoH(out, g_s.dti, 8), "dti readback");
}

int refh_temperature_floor(unsigned long long U_, int nx, int ny, int nz, int ng, int nf, double U_floor)
{
  return launch(K_TFLOOR, (size_t)nx * ny * nz, (CUdeviceptr)U_, nx, ny, nz, ng, nf, U_floor);
}

// Grid3D::Set_Boundaries for the six faces in order (boundary_conditions.cpp:54-131, 412-500).
int refh_set_boundaries(unsigned long long U_, int nx, int ny, int nz, int ng, int nf, const int *flags)
{
  CUdeviceptr U = (CUdeviceptr)U_;
  int f[6];
  for (int i = 0; i < 6; i++) f[i] = flags[i];
  int const n_cells = nx * ny * nz;
  for (int dir = 0; dir < 6; dir++) {
    if ((dir < 2 && nx <= 1) || (dir >= 2 && dir < 4 && ny <= 1) || (dir >= 4 && nz <= 1)) continue;
    if (f[dir] == 4) continue;
    int jl = 0, ju = ny, kl = 0, ku = nz;
    if (ny > 1) jl = ng, ju = ny - ng;
    if (nz > 1) kl = ng, ku = nz - ng;
    int imin[3], imax[3];
    if (dir == 0) imin[0] = 0, imax[0] = ng, imin[1] = jl, imax[1] = ju, imin[2] = kl, imax[2] = ku;
    if (dir == 1) imin[0] = nx - ng, imax[0] = nx, imin[1] = jl, imax[1] = ju, imin[2] = kl, imax[2] = ku;
    if (dir == 2) imin[0] = 0, imax[0] = nx, imin[1] = 0, imax[1] = ng, imin[2] = kl, imax[2] = ku;
    if (dir == 3) imin[0] = 0, imax[0] = nx, imin[1] = ny - ng, imax[1] = ny, imin[2] = kl, imax[2] = ku;
    if (dir == 4) imin[0] = 0, imax[0] = nx, imin[1] = 0, imax[1] = ny, imin[2] = 0, imax[2] = ng;
    if (dir == 5) imin[0] = 0, imax[0] = nx, imin[1] = 0, imax[1] = ny, imin[2] = nz - ng, imax[2] = nz;
    int const is = imax[0] - imin[0], js = imax[1] - imin[1], ks = imax[2] - imin[2];
    if (launch(K_GHOST, (size_t)is * js * ks, U, nx, ny, nz, nf, n_cells, ng, f[0], f[1], f[2], f[3], f[4], f[5], is,
               js, ks, imin[0], imin[1], imin[2], dir))
      return 1;
  }
  return 0;
}

int refh_sync(void) { return cu(cuStreamSynchronize(g_stream), "sync"); }

// 1: synchronise the context after every kernel, as the reference's default build does
int refh_set_sync_each(int on)
{
  g_sync_each = on != 0;
  return 0;
}

int refh_free(void)
{
  free_scratch();
  return 0;
}

}  // extern "C"
