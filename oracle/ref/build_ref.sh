#!/bin/bash
# Builds the reference xcorr-gpu from its own sources, unchanged, into
# oracle/_ref/ (git-ignored).  Two programs come out:
#   oracle/_ref/xcorr-gpu       the reference as its Makefile builds it
#   oracle/_ref/xcorr-gpu-dump  the same objects plus oracle/ref/dump_hooks.cu,
#                               which records per-location results at full precision
# and oracle/_ref/ref_host_probe, the reference's host C functions (PRM parse,
# location grid, result writer) behind a small driver for CPU parity tests, and
# oracle/_ref/ref_time_probe, the reference's do_time_corr (-time / -time4) on
# supplied integer patches, and oracle/_ref/xcorr-gb300-shim, the reference
# program calling this library in place of its do_correlation.
#
# Two additions are needed for a current toolchain (both outside the sources):
#   * oracle/ref/helper_cuda.h stands in for the CUDA-samples header named in gpu_err.h:9;
#   * -fcommon, because gmtsar_d.h:60-71 defines globals in a header.
# The hook renames are -D flags on the calling translation units only.
#
# usage: oracle/ref/build_ref.sh REFERENCE_SOURCE_DIR [--host-only]
set -euo pipefail
REF=${1:?usage: build_ref.sh REFERENCE_SOURCE_DIR [--host-only]}
MODE=${2:-all}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$(cd "$HERE/.." && pwd)/_ref
OBJ=$OUT/obj
mkdir -p "$OBJ"
[ -f "$REF/xcorr.cu" ] || { echo "build_ref: no reference sources in $REF" >&2; exit 2; }

CC=${CC:-gcc}
CFLAGS="-O2 -Wall -fPIC -fno-strict-aliasing -std=c99 -fcommon -I$REF -w"
for f in print_results get_locations parse_xcorr_input utils read_xcorr_data sio_struct plxyz; do
  $CC $CFLAGS -c "$REF/$f.c" -o "$OBJ/$f.o" &
done
$CC $CFLAGS -Dprint_results=xcg_ref_orig_print_results -c "$REF/print_results.c" -o "$OBJ/print_results_renamed.o" &
wait

# host-side probe: reference parse/locations/writer driven from argv
$CC -O2 -std=c99 -fcommon -w -I"$REF" "$HERE/ref_host_probe.c" \
    "$OBJ/get_locations.o" "$OBJ/parse_xcorr_input.o" "$OBJ/utils.o" "$OBJ/sio_struct.o" \
    "$OBJ/print_results.o" "$OBJ/read_xcorr_data.o" "$OBJ/plxyz.o" -lm -o "$OUT/ref_host_probe"
[ "$MODE" = "--host-only" ] && { echo "build_ref: host probe in $OUT"; exit 0; }

NVCC=${NVCC:-nvcc}
NV="$NVCC -I$HERE -I$REF -w"
$NV -c "$REF/xcorr.cu" -o "$OBJ/xcorr.o" &
$NV -c "$REF/fft_interpolate_routines.cu" -o "$OBJ/fft_interpolate_routines.o" &
$NV -maxrregcount 36 -c "$REF/conv_ampl_demean.cu" -o "$OBJ/conv_ampl_demean.o" &
$NV -c "$REF/do_freq_xcorr.cu" -o "$OBJ/do_freq_xcorr.o" &
$NV -c "$REF/do_time_int_xcorr.cu" -o "$OBJ/do_time_int_xcorr.o" &
$NV -c "$REF/highres_corr.cu" -o "$OBJ/highres_corr.o" &
# dump variants of the calling units
$NV -Dh_reduceFD_strip=xcg_hook_h_reduceFD_strip -c "$REF/xcorr.cu" -o "$OBJ/xcorr_dump.o" &
$NV -Dh_reduce_strip=xcg_hook_h_reduce_strip -c "$REF/do_freq_xcorr.cu" -o "$OBJ/do_freq_xcorr_dump.o" &
$NV -Dh_reduceCr_strip=xcg_hook_h_reduceCr_strip -c "$REF/highres_corr.cu" -o "$OBJ/highres_corr_dump.o" &
$NV -c "$HERE/dump_hooks.cu" -o "$OBJ/dump_hooks.o" &
wait

# time-domain probe: the reference's do_time_corr on supplied integer patches
$CC -O2 -std=c99 -fcommon -w -I"$REF" -c "$HERE/ref_time_probe.c" -o "$OBJ/ref_time_probe.o"
$NVCC "$OBJ/ref_time_probe.o" "$OBJ/do_time_int_xcorr.o" "$OBJ/conv_ampl_demean.o" "$OBJ/utils.o" "$OBJ/plxyz.o" \
      -lm -o "$OUT/ref_time_probe"

LIBC="$OBJ/get_locations.o $OBJ/parse_xcorr_input.o $OBJ/utils.o $OBJ/read_xcorr_data.o $OBJ/sio_struct.o $OBJ/plxyz.o"
$NVCC "$OBJ/xcorr.o" "$OBJ/fft_interpolate_routines.o" "$OBJ/conv_ampl_demean.o" "$OBJ/do_freq_xcorr.o" \
      "$OBJ/do_time_int_xcorr.o" "$OBJ/highres_corr.o" $LIBC "$OBJ/print_results.o" -lm -lcufft -o "$OUT/xcorr-gpu"
$NVCC "$OBJ/xcorr_dump.o" "$OBJ/fft_interpolate_routines.o" "$OBJ/conv_ampl_demean.o" "$OBJ/do_freq_xcorr_dump.o" \
      "$OBJ/do_time_int_xcorr.o" "$OBJ/highres_corr_dump.o" "$OBJ/dump_hooks.o" $LIBC "$OBJ/print_results_renamed.o" \
      -lm -lcufft -o "$OUT/xcorr-gpu-dump"
# the reference program with its do_correlation replaced by the library call
# of gmtsar-gpu_gb300/integration/do_correlation_shim.cpp (the binding
# INTEGRATION.md shows): xcorr.cu's host code compiled without inlining and
# its do_correlation made a weak symbol, so main, set_defaults,
# parse_command_line, handle_prm, get_locations and print_results are the
# reference's own and main calls the shim's definition
PKGDIR=$(cd "$HERE/../../gmtsar-gpu_gb300" && pwd)
if [ -f "$PKGDIR/lib/libxcorr_gb300.so" ]; then
  $NV -Xcompiler -O0 -Xcompiler -fno-inline -c "$REF/xcorr.cu" -o "$OBJ/xcorr_shimhost.o"
  # do_correlation(struct xcorr) with C++ linkage, as xcorr.cu (CUDA C++) defines it
  objcopy --weaken-symbol=_Z14do_correlation5xcorr "$OBJ/xcorr_shimhost.o"
  ${CXX:-g++} -O2 -fcommon -w -I"$REF" -I"$PKGDIR/../include" -c "$PKGDIR/integration/do_correlation_shim.cpp" \
      -o "$OBJ/do_correlation_shim.o"
  $NVCC "$OBJ/xcorr_shimhost.o" "$OBJ/do_correlation_shim.o" "$OBJ/fft_interpolate_routines.o" \
        "$OBJ/conv_ampl_demean.o" "$OBJ/do_freq_xcorr.o" "$OBJ/do_time_int_xcorr.o" "$OBJ/highres_corr.o" $LIBC \
        "$OBJ/print_results.o" -L"$PKGDIR/lib" -lxcorr_gb300 -Xlinker -rpath -Xlinker "$PKGDIR/lib" -lm -lcufft \
        -o "$OUT/xcorr-gb300-shim"
fi
echo "build_ref: built $OUT/xcorr-gpu $OUT/xcorr-gpu-dump $OUT/ref_host_probe $OUT/ref_time_probe $OUT/xcorr-gb300-shim"
