#!/usr/bin/env bash
# Builds the reference HiQ state-vector engine (_cppsim_mpi) and cluster
# scheduler (_sched_cpp) from their sources, unmodified, as single-rank CPU
# oracles, against the stand-in headers in oracle/shim/. Output goes to
# oracle/_ref/ only (git-ignored). Needs the reference sources (argument 1 or
# $HIQ_REFERENCE_SRC, default /root/reference) and pybind11 headers; when
# either is absent it prints why and exits 0 without building.
#
#   REF_FLAGS  extra compiler flags; default "-O2 -fopenmp" (parity build).
#              The reference's release flags are "-O3 -ffast-math -march=native".
#   REF_VARIANT  build into oracle/_ref/<variant>/ instead (e.g. "release" with
#              REF_FLAGS="-O3 -ffast-math -fopenmp" for timing the reference's
#              own kernels beside the oracle port).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${1:-${HIQ_REFERENCE_SRC:-/root/reference}}"
OUT="$HERE/_ref${REF_VARIANT:+/$REF_VARIANT}"
case "${REF_VARIANT:-}" in */*|..*) echo "build_ref: REF_VARIANT must be a plain name"; exit 1;; esac
FLAGS="${REF_FLAGS:--O2 -fopenmp}"
if [ ! -f "$SRC/src/simulator-mpi/SimulatorMPI.cpp" ]; then
    echo "build_ref: reference sources not found at $SRC; skipped"; exit 0
fi
PYBIND_INC="$(python3 -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || true)"
if [ -z "$PYBIND_INC" ]; then
    TORCH_INC="$(python3 -c 'import torch, os; print(os.path.join(os.path.dirname(torch.__file__), "include"))' 2>/dev/null || true)"
    [ -d "$TORCH_INC/pybind11" ] && PYBIND_INC="$TORCH_INC"
fi
if [ -z "$PYBIND_INC" ]; then echo "build_ref: no pybind11 headers; skipped"; exit 0; fi
PY_INC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
ARCH="$(uname -m)"
KFLAG="-DNOINTRIN"
mkdir -p "$OUT"
CXX="${CXX:-g++}"
COMMON="-std=c++17 -shared -fPIC $FLAGS $KFLAG -I$HERE/shim -I$SRC/src -I$PYBIND_INC -I$PY_INC -w"
$CXX $COMMON -o "$OUT/_cppsim_mpi$EXT" "$SRC/_cppsim_mpi.cpp" \
    "$SRC/src/simulator-mpi/SimulatorMPI.cpp" "$SRC/src/simulator-mpi/SwapperMT.cpp" \
    "$SRC/src/simulator-mpi/funcs.cpp" -lpthread &
$CXX $COMMON -o "$OUT/_sched_cpp$EXT" "$SRC/_sched_cpp.cpp" \
    "$SRC/src/scheduler/cluster_scheduler.cpp" "$SRC/src/scheduler/swap_scheduler.cpp" \
    "$SRC/src/scheduler/convertors.cpp" &
wait %1 && wait %2
echo "build_ref: built $OUT/_cppsim_mpi$EXT and $OUT/_sched_cpp$EXT ($ARCH, $KFLAG, $FLAGS)"
