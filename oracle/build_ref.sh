#!/usr/bin/env bash
# Compile the reference's own hot-path CUDA kernels (unchanged, from the cholla source tree)
# into device-only cubins under oracle/_ref/<variant>/, with the reference Makefile's device
# flags (Makefile:70,148: -O3 -std=c++17 --expt-extended-lambda -fmad=false) for sm_103a.
# The cubins are test infrastructure: oracle/ref_harness.cpp loads them with the CUDA driver
# API to run the reference's VL step on the GPU as the parity and speed baseline.
# Usage: oracle/build_ref.sh /path/to/cholla
set -euo pipefail
REF=${1:-${CHOLLA_REFERENCE:-$(cd "$(dirname "$0")/../.." && pwd)/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
FLAGS="-O3 -std=c++17 --expt-extended-lambda -fmad=false -gencode arch=compute_103a,code=sm_103a -cubin -I$REF/src"
COMMON="-DVL -DPRECISION=2 -DDENSITY_FLOOR -DTEMPERATURE_FLOOR"
# The reference's VL integrators do not compile with the exact solver (integrators/VL_3D_cuda.cu:149
# runs the argument n_cells into the kernel's name); the harness uses only their update kernels,
# which no solver macro changes, so in the exact variant they are compiled with -DHLLC instead.
declare -A DEFS=(
  [hydro_ppmc_hllc_de]="$COMMON -DPPMC -DHLLC -DDE"
  [hydro_ppmc_hllc]="$COMMON -DPPMC -DHLLC"
  [hydro_plmc_hllc]="$COMMON -DPLMC -DHLLC"
  [hydro_ppmc_roe_de]="$COMMON -DPPMC -DROE -DDE"
  [hydro_ppmc_hll_de]="$COMMON -DPPMC -DHLL -DDE"
  [mhd_plmc_hlld]="$COMMON -DPLMC -DHLLD -DMHD"
  [hydro_plmp_hllc]="$COMMON -DPLMP -DHLLC"
  [hydro_ppmp_hll_de]="$COMMON -DPPMP -DHLL -DDE"
  [hydro_ppmc_exact_de]="$COMMON -DPPMC -DEXACT -DDE"
)
declare -A FILES=(
  [hydro]="integrators/VL_3D_cuda.cu integrators/VL_1D_cuda.cu hydro/hydro_cuda.cu reconstruction/pcm_cuda.cu reconstruction/ppmc_cuda.cu reconstruction/plmc_cuda.cu reconstruction/plmp_cuda.cu reconstruction/ppmp_cuda.cu riemann_solvers/hllc_cuda.cu riemann_solvers/roe_cuda.cu riemann_solvers/hll_cuda.cu riemann_solvers/exact_cuda.cu grid/cuda_boundaries.cu"
  [mhd]="integrators/VL_3D_cuda.cu hydro/hydro_cuda.cu reconstruction/pcm_cuda.cu reconstruction/plmc_cuda.cu riemann_solvers/hlld_cuda.cu mhd/ct_electric_fields.cu mhd/magnetic_update.cu mhd/magnetic_divergence.cu grid/cuda_boundaries.cu"
)
pids=()
for v in "${!DEFS[@]}"; do
  mkdir -p "$OUT/$v"
  kind=${v%%_*}
  for f in ${FILES[$kind]}; do
    o="$OUT/$v/$(basename "$f" .cu).cubin"
    if [[ ! -f "$o" || "$REF/src/$f" -nt "$o" || "$0" -nt "$o" ]]; then
      defs=${DEFS[$v]}
      if [[ $f == integrators/* ]]; then defs=${defs/-DEXACT/-DHLLC}; fi
      $NVCC $FLAGS $defs "$REF/src/$f" -o "$o" &
      pids+=($!)
    fi
  done
done
for p in "${pids[@]}"; do wait "$p"; done
echo "reference cubins in $OUT"
