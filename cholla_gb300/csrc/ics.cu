// ics.cu -- initial conditions written on the device: a spherical blast and a shock tube of any
// orientation (the problems of the serving workload).  Every cell of the padded box is set, the
// ghosts included.
#include <cuda_runtime.h>

#include "../../include/cholla_gb300.h"
#include "common.cuh"

namespace
{
struct IC {
  int nx, ny, nz, ng, nf, de;
  double dx, dy, dz, gamma;
  double cx, cy, cz;
  int kind;          // 0 blast, 1 shock tube
  double radius, e_in, rho, p;          // blast
  double nxv, nyv, nzv, rl, pl, rr, pr;  // tube
};

__global__ void k_ic(IC c, double *__restrict__ U)
{
  long long const n = (long long)c.nx * c.ny * c.nz;
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < n;
       id += (long long)gridDim.x * blockDim.x) {
    int const z = (int)(id / ((long long)c.nx * c.ny));
    int const y = (int)((id / c.nx) % c.ny);
    int const x = (int)(id % c.nx);
    double const px = (x - c.ng + 0.5) * c.dx - c.cx, py = (y - c.ng + 0.5) * c.dy - c.cy,
                 pz = (z - c.ng + 0.5) * c.dz - c.cz;
    double d, e;  // density, internal energy per volume
    if (c.kind == 0) {
      d = c.rho;
      e = c.p / (c.gamma - 1.0);
      if (px * px + py * py + pz * pz < c.radius * c.radius) e += c.e_in;
    } else {
      bool const left = px * c.nxv + py * c.nyv + pz * c.nzv < 0.0;
      d = left ? c.rl : c.rr;
      e = (left ? c.pl : c.pr) / (c.gamma - 1.0);
    }
    U[id]         = d;
    U[n + id]     = 0.0;
    U[2 * n + id] = 0.0;
    U[3 * n + id] = 0.0;
    U[4 * n + id] = e;
    for (int f = 5; f < c.nf; f++) U[(long long)f * n + id] = 0.0;
    if (c.de) U[(long long)(c.nf - 1) * n + id] = e;
  }
}

int launch(const IC &c, double *U, void *stream)
{
  if (!U || c.nx < 1 || c.ny < 1 || c.nz < 1 || c.nf < 5 || !(c.gamma > 1.0)) return CGB_ERR_ARGS;
  long long const n = (long long)c.nx * c.ny * c.nz;
  long long blocks  = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_ic<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(c, U);
  return cudaGetLastError() == cudaSuccess ? CGB_OK : CGB_ERR_CUDA;
}
}  // namespace

extern "C" {

int cgb_ic_blast(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx, double dy,
                 double dz, double cx, double cy, double cz, double radius, double energy, double rho, double p,
                 double gamma, int dual_energy, void *stream)
{
  if (!(radius > 0)) return CGB_ERR_ARGS;
  // thermal energy per volume inside the sphere, from the volume of the cells it covers
  int const rx = nx - 2 * n_ghost, ry = ny - 2 * n_ghost, rz = nz - 2 * n_ghost;
  long long inside = 0;
  for (int z = 0; z < rz; z++)
    for (int y = 0; y < ry; y++)
      for (int x = 0; x < rx; x++) {
        double const px = (x + 0.5) * dx - cx, py = (y + 0.5) * dy - cy, pz = (z + 0.5) * dz - cz;
        if (px * px + py * py + pz * pz < radius * radius) inside++;
      }
  if (inside == 0) return CGB_ERR_ARGS;
  IC c{};
  c.nx = nx, c.ny = ny, c.nz = nz, c.ng = n_ghost, c.nf = n_fields, c.de = dual_energy ? 1 : 0;
  c.dx = dx, c.dy = dy, c.dz = dz, c.gamma = gamma, c.cx = cx, c.cy = cy, c.cz = cz;
  c.kind = 0, c.radius = radius, c.e_in = energy / (inside * dx * dy * dz), c.rho = rho, c.p = p;
  return launch(c, d_conserved, stream);
}

int cgb_ic_shock_tube(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx, double dy,
                      double dz, double cx, double cy, double cz, double nxv, double nyv, double nzv, double rho_l,
                      double p_l, double rho_r, double p_r, double gamma, int dual_energy, void *stream)
{
  IC c{};
  c.nx = nx, c.ny = ny, c.nz = nz, c.ng = n_ghost, c.nf = n_fields, c.de = dual_energy ? 1 : 0;
  c.dx = dx, c.dy = dy, c.dz = dz, c.gamma = gamma, c.cx = cx, c.cy = cy, c.cz = cz;
  c.kind = 1, c.nxv = nxv, c.nyv = nyv, c.nzv = nzv, c.rl = rho_l, c.pl = p_l, c.rr = rho_r, c.pr = p_r;
  return launch(c, d_conserved, stream);
}

}  // extern "C"
