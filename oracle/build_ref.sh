#!/usr/bin/env bash
# Builds oracle/_ref/libnoa_ref_dcs.so: the reference's own src/noa/pms/dcs.hh
# (read in place from the noa checkout, never copied) behind the C wrapper
# oracle/ref_dcs_wrapper.cc, against the pip LibTorch.  Test infrastructure
# only.  Usage: oracle/build_ref.sh [NOA_CHECKOUT]   (default /root/reference)
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
noa="${1:-/root/reference}"
if [ ! -f "$noa/src/noa/pms/dcs.hh" ]; then
    echo "build_ref.sh: no noa checkout at $noa; skipping" >&2
    exit 0
fi
torch_dir="$(python3 -c 'import os, torch; print(os.path.dirname(torch.__file__))')"
mkdir -p "$here/_ref"
g++ -std=c++20 -O3 -fopenmp -fPIC -shared -D_GLIBCXX_USE_CXX11_ABI=1 \
    -I"$noa/src" -I"$torch_dir/include" -I"$torch_dir/include/torch/csrc/api/include" \
    "$here/ref_dcs_wrapper.cc" -o "$here/_ref/libnoa_ref_dcs.so" \
    -L"$torch_dir/lib" -Wl,-rpath,"$torch_dir/lib" -ltorch -ltorch_cpu -lc10
echo "built $here/_ref/libnoa_ref_dcs.so"
