// ghost.cuh -- ghost-cell fill of one cell of a padded box (single GPU, no MPI faces).
//
// Same mapping as the reference's SetGhostCellsKernel / SetBoundaryMapping / FindIndex
// (src/grid/cuda_boundaries.cu:71-300) with the face extents of Set_Boundary_Extents
// (src/grid/boundary_conditions.cpp:412-500).  The reference fills the six faces in six
// launches; every ghost cell reads a real cell, so one pass over all ghost cells, each cell
// taking the face whose launch would have written it last (z, then y, then x), gives the
// same result.
#pragma once
#include "common.cuh"

namespace cgb
{

static __device__ __forceinline__ int ghost_find_index(int ig, int nx, int flag, int face, int ng, double *a)
{
  if (face == 0) {
    switch (flag) {
      case 1: return ig + nx - 2 * ng;               // periodic
      case 2: *a = -1.0; return 2 * ng - ig - 1;     // reflective
      case 3: return ng;                              // transmissive
      case 4: return -1;                              // custom: left alone
      case 5: return ig;                              // exchanged elsewhere: left alone
      default: return ig + nx - 2 * ng;
    }
  }
  switch (flag) {
    case 1: return ig - nx + 2 * ng;
    case 2: *a = -1.0; return 2 * (nx - ng) - ig - 1;
    case 3: return nx - ng - 1;
    case 4: return -1;
    case 5: return ig;
    default: return ig - nx + 2 * ng;
  }
}

struct Flags {
  int f[6];
};

// fl.f: boundary flag per face, 0 for a dimension of extent 1 (ghost_flags)
static __device__ __forceinline__ void ghost_cell(const Box &b, double *__restrict__ U, const Flags &fl, long long id)
{
  int const ng = b.ng, nx = b.nx, ny = b.ny, nz = b.nz;
  int const k = (int)(id / ((long long)nx * ny));
  int const j = (int)((id - (long long)k * nx * ny) / nx);
  int const i = (int)(id - (long long)k * nx * ny - (long long)j * nx);
  bool const gx = nx > 1 && (i < ng || i >= nx - ng);
  bool const gy = ny > 1 && (j < ng || j >= ny - ng);
  bool const gz = nz > 1 && (k < ng || k >= nz - ng);
  if (!(gx || gy || gz)) return;
  // the face whose launch owns this cell
  int dir = gz ? (k < ng ? 4 : 5) : gy ? (j < ng ? 2 : 3) : (i < ng ? 0 : 1);
  if (fl.f[dir] == 4 || fl.f[dir] == 5) return;
  double a[3] = {1., 1., 1.};
  long long idx = 0;
  int r;
  if (nx > 1) {
    r = (i < ng) ? ghost_find_index(i, nx, fl.f[0], 0, ng, &a[0]) : (i >= nx - ng) ? ghost_find_index(i, nx, fl.f[1], 1, ng, &a[0]) : i;
    if (r < 0) return;
    idx += r;
  }
  if (ny > 1) {
    r = (j < ng) ? ghost_find_index(j, ny, fl.f[2], 0, ng, &a[1]) : (j >= ny - ng) ? ghost_find_index(j, ny, fl.f[3], 1, ng, &a[1]) : j;
    if (r < 0) return;
    idx += (long long)nx * r;
  }
  if (nz > 1) {
    r = (k < ng) ? ghost_find_index(k, nz, fl.f[4], 0, ng, &a[2]) : (k >= nz - ng) ? ghost_find_index(k, nz, fl.f[5], 1, ng, &a[2]) : k;
    if (r < 0) return;
    idx += (long long)nx * ny * r;
  }
  long long const n = b.n;
  for (int f = 0; f < b.nf; f++) U[id + f * n] = U[idx + f * n];
  if (fl.f[0] == 2 || fl.f[1] == 2) U[id + n] *= a[0];
  if (fl.f[2] == 2 || fl.f[3] == 2) U[id + 2 * n] *= a[1];
  if (fl.f[4] == 2 || fl.f[5] == 2) U[id + 3 * n] *= a[2];
  if (!b.mhd && fl.f[dir] == 3) {
    // diode: no inflow through a transmissive face (cuda_boundaries.cu:120-146)
    long long const momdex = id + (long long)(dir / 2 + 1) * n;
    if ((dir % 2 == 0) ? (U[momdex] > 0.0) : (U[momdex] < 0.0)) {
      U[id + 4 * n] -= 0.5 * (U[momdex] * U[momdex]) / U[id];
      U[momdex] = 0.0;
    }
  }
}

inline Flags ghost_flags(const Box &b, const int flags[6])
{
  Flags fl;
  for (int i = 0; i < 6; i++) fl.f[i] = flags[i];
  if (b.nx <= 1) fl.f[0] = fl.f[1] = 0;
  if (b.ny <= 1) fl.f[2] = fl.f[3] = 0;
  if (b.nz <= 1) fl.f[4] = fl.f[5] = 0;
  return fl;
}
}  // namespace cgb
