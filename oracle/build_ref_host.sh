#!/usr/bin/env bash
# Compile the reference's own VL integrators and hot-path kernels, unchanged from the cholla
# source tree, as host C++ (oracle/ref_host_shim.h + oracle/ref_host.cpp): one shared library per
# scheme under oracle/_ref/host/<variant>.so.  Test infrastructure: the CPU suite runs the
# reference itself through these to pin the FP64 restatement bit for bit without a GPU.
# -ffp-contract=off is the host counterpart of the reference Makefile's -fmad=false (Makefile:70).
# Usage: oracle/build_ref_host.sh /path/to/cholla
set -euo pipefail
REF=${1:-${CHOLLA_REFERENCE:-$(cd "$(dirname "$0")/../.." && pwd)/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref/host"
CXX=${CXX:-g++}
CUDA_HOME=${CUDA_HOME:-/usr/local/cuda}
FLAGS="-std=c++17 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared -w -I$CUDA_HOME/include -I$REF/src -include $HERE/ref_host_shim.h"
COMMON="-DVL -DPRECISION=2 -DDENSITY_FLOOR -DTEMPERATURE_FLOOR"
# The exact-solver libraries hold its flux kernel but no integrator: the reference's VL
# integrators do not compile with -DEXACT (integrators/VL_3D_cuda.cu:149 runs the argument
# n_cells into the kernel's name).
declare -A DEFS=(
  [pcm_exact]="-DPCM -DEXACT"
  [pcm_exact_de]="-DPCM -DEXACT -DDE"
  [ppmc_hllc_de]="-DPPMC -DHLLC -DDE"
  [ppmc_hllc]="-DPPMC -DHLLC"
  [ppmc_hllc_de_scalar]="-DPPMC -DHLLC -DDE -DSCALAR -DBASIC_SCALAR"
  [plmc_hllc]="-DPLMC -DHLLC"
  [pcm_hllc_de]="-DPCM -DHLLC -DDE"
  [ppmc_roe_de]="-DPPMC -DROE -DDE"
  [ppmc_hll_de]="-DPPMC -DHLL -DDE"
  [plmp_hllc]="-DPLMP -DHLLC"
  [plmp_hllc_de]="-DPLMP -DHLLC -DDE"
  [plmp_hll]="-DPLMP -DHLL"
  [ppmp_hllc_de]="-DPPMP -DHLLC -DDE"
  [ppmp_hllc]="-DPPMP -DHLLC"
  [ppmp_roe]="-DPPMP -DROE"
  [mhd_plmc_hlld]="-DPLMC -DHLLD -DMHD"
  [mhd_ppmc_hlld]="-DPPMC -DHLLD -DMHD"
)
mkdir -p "$OUT"
pids=()
for v in "${!DEFS[@]}"; do
  o="$OUT/$v.so"
  if [[ ! -f "$o" || "$HERE/ref_host.cpp" -nt "$o" || "$HERE/ref_host_shim.h" -nt "$o" || "$0" -nt "$o" ]]; then
    $CXX $FLAGS $COMMON ${DEFS[$v]} "$HERE/ref_host.cpp" -o "$o" &
    pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
echo "host-compiled reference in $OUT"
