#!/usr/bin/env bash
# Builds the reference's own code for the parity and baseline legs.  Test and
# benchmark infrastructure only: nothing here is linked into the product.
#
#   oracle/_ref/libnoa_ref_dcs.so   src/noa/pms/dcs.hh on the CPU (dcs::vmap,
#                                   dcs::pvmap with OpenMP, -O3), behind
#                                   oracle/ref_dcs_wrapper.cc, without FMA
#                                   contraction: the parity build, bit for bit
#                                   the x86-64 build that made tests/golden
#   oracle/_ref/libnoa_ref_dcs_bench.so  the same with the reference benchmark's
#                                   own flags (benchmark/CMakeLists.txt:33-37:
#                                   -O3, OpenMP, the compiler's default
#                                   contraction, which fuses a*b+c on aarch64):
#                                   the timed CPU baseline
#   oracle/_ref/libnoa_ref_cuda.so  src/noa/pms/dcs.cuh, the reference's one CUDA
#                                   kernel (dcs::cuda::vmap_bremsstrahlung), for
#                                   sm_103a, behind oracle/ref_cuda_wrapper.cu
#   oracle/_ref/ref_dropin_caller   oracle/ref_dropin_caller.cc, a program written
#                                   against the reference's declarations only,
#                                   linked with noa_gb300/libnoa_dcs_torch.so
#                                   (stage "caller"; needs that library built)
#
# Sources.  The six reference headers the path needs are staged UNMODIFIED from
# the noa checkout (NOA_CHECKOUT, else the build container's checkout) into
# oracle/_ref/src.  That folder is git-ignored and never committed; it travels
# with the working tree to a GPU host that has no checkout, which then builds
# from the staged copy.  Where neither exists the script does nothing.
#
# Usage: oracle/build_ref.sh [all|caller]
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(dirname "$here")"
stage="${1:-all}"
noa="${NOA_CHECKOUT:-/root/reference}"
out="$here/_ref"
src="$out/src"
headers="noa/pms/dcs.hh noa/pms/dcs.cuh noa/pms/physics.hh noa/utils/common.hh noa/utils/common.cuh noa/utils/numerics.hh"

if [ -f "$noa/src/noa/pms/dcs.hh" ]; then
    for f in $headers; do
        mkdir -p "$src/$(dirname "$f")"
        cp -pf "$noa/src/$f" "$src/$f"
    done
fi
if [ ! -f "$src/noa/pms/dcs.hh" ]; then
    echo "build_ref.sh: no noa checkout and no staged reference sources; skipping" >&2
    exit 0
fi

torch_dir="$(python3 -c 'import os, torch; print(os.path.dirname(torch.__file__))')"
abi="$(python3 -c 'import torch; print(int(bool(torch._C._GLIBCXX_USE_CXX11_ABI)))')"
nvcc="$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)"
tinc=(-I"$torch_dir/include" -I"$torch_dir/include/torch/csrc/api/include")
tlib=(-L"$torch_dir/lib" -Wl,-rpath,"$torch_dir/lib")
tlib_nvcc=(-L"$torch_dir/lib" -Xlinker -rpath -Xlinker "$torch_dir/lib")

newer() {  # newer TARGET DEPS...: true when TARGET is missing or older than a dependency
    local t="$1"; shift
    [ -f "$t" ] || return 0
    for d in "$@"; do [ "$d" -nt "$t" ] && return 0; done
    return 1
}

mkdir -p "$out"
staged=()
for f in $headers; do staged+=("$src/$f"); done

if [ "$stage" = "all" ]; then
    pids=()
    # the reference's CMake: C++20, OpenMP, -O3 (CMakeLists.txt:34-39,
    # benchmark/CMakeLists.txt:33-37)
    for variant in parity bench; do
        if [ "$variant" = parity ]; then lib="$out/libnoa_ref_dcs.so"; fpc=(-ffp-contract=off)
        else lib="$out/libnoa_ref_dcs_bench.so"; fpc=(); fi
        if newer "$lib" "$here/ref_dcs_wrapper.cc" "${staged[@]}"; then
            g++ -std=c++20 -O3 -fopenmp -fPIC -shared "${fpc[@]}" -D_GLIBCXX_USE_CXX11_ABI="$abi" \
                -I"$src" "${tinc[@]}" "$here/ref_dcs_wrapper.cc" -o "$lib" \
                "${tlib[@]}" -ltorch -ltorch_cpu -lc10 &
            pids+=($!)
        fi
    done
    if newer "$out/libnoa_ref_cuda.so" "$here/ref_cuda_wrapper.cu" "${staged[@]}"; then
        # the reference's CUDA flags: C++17, --expt-relaxed-constexpr
        # --expt-extended-lambda (CMakeLists.txt:49, 65).  -Bsymbolic binds the
        # wrapper's call to the reference's own vmap_bremsstrahlung, never to
        # the drop-in's definition of the same mangled name in a process that
        # has loaded both.
        "$nvcc" -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 --expt-relaxed-constexpr \
            --expt-extended-lambda -Xcompiler -fPIC -shared -D_GLIBCXX_USE_CXX11_ABI="$abi" \
            -I"$src" "${tinc[@]}" "$here/ref_cuda_wrapper.cu" -o "$out/libnoa_ref_cuda.so" \
            -Xlinker -Bsymbolic "${tlib_nvcc[@]}" -ltorch -ltorch_cpu -lc10 -ltorch_cuda -lc10_cuda &
        pids+=($!)
    fi
    rc=0
    for p in "${pids[@]}"; do wait "$p" || rc=1; done
    exit $rc
fi

if [ "$stage" = "caller" ]; then
    pkg="$root/noa_gb300"
    if [ ! -f "$pkg/libnoa_dcs_torch.so" ]; then
        echo "build_ref.sh: noa_gb300/libnoa_dcs_torch.so not built; skipping the drop-in caller" >&2
        exit 0
    fi
    if newer "$out/ref_dropin_caller" "$here/ref_dropin_caller.cc" "$pkg/libnoa_dcs_torch.so" "${staged[@]}"; then
        # Include path: the staged reference sources and LibTorch only, never
        # this repository's include/, so the declarations are the reference's.
        g++ -std=c++20 -O2 -D_GLIBCXX_USE_CXX11_ABI="$abi" -I"$src" "${tinc[@]}" \
            "$here/ref_dropin_caller.cc" -o "$out/ref_dropin_caller" \
            -L"$pkg" -Wl,-rpath,'$ORIGIN/../../noa_gb300' -lnoa_dcs_torch -lnoa_dcs \
            "${tlib[@]}" -ltorch -ltorch_cpu -lc10 -ltorch_cuda -lc10_cuda
    fi
    exit 0
fi
echo "build_ref.sh: unknown stage $stage" >&2
exit 2
