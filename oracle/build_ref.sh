#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.  Builds the UNMODIFIED reference C++ sources, read
# in place from the read-only reference checkout, into oracle/_ref/libwndref.so
# (git-ignored).  Added here: a 4-define config.h and a libtiff stand-in header
# (oracle/ref_shim/include), the FFTW3 shim (oracle/ref_shim/fftw_shim.cpp) and
# the C ABI used by the tests (oracle/ref_shim/ref_capi.cpp).
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# VARIANT=fma builds a second copy into oracle/_ref_fma/ with floating-point
# contraction into fused multiply-adds (x86-64: -mfma; aarch64 contracts by
# default): the reference as a contracting compiler builds it, used to measure
# the reference's own build-to-build spread on rounding-sensitive features.
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
VARIANT="${VARIANT:-}"
OUT="$HERE/_ref${VARIANT:+_$VARIANT}"
SRC="$REF/src"
if [ ! -d "$SRC" ]; then echo "reference sources not found at $SRC" >&2; exit 2; fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS="-O2 -fPIC -w -std=gnu++11 -I$HERE/ref_shim/include -I$SRC"
if [ "$VARIANT" = "fma" ]; then
  case "$(uname -m)" in x86_64) FLAGS="$FLAGS -mfma -ffp-contract=fast" ;; *) FLAGS="$FLAGS -ffp-contract=fast" ;; esac
fi
FILES="cmatrix.cpp FeatureAlgorithms.cpp FeatureNames.cpp ImageTransforms.cpp Tasks.cpp wndchrm_error.cpp
transforms/ChebyshevFourier.cpp transforms/chebyshev.cpp transforms/radon.cpp
transforms/wavelet/Common.cpp transforms/wavelet/DataGrid2D.cpp transforms/wavelet/DataGrid3D.cpp
transforms/wavelet/Filter.cpp transforms/wavelet/FilterSet.cpp transforms/wavelet/Symlet5.cpp
transforms/wavelet/Wavelet.cpp transforms/wavelet/WaveletHigh.cpp transforms/wavelet/WaveletLow.cpp
transforms/wavelet/WaveletMedium.cpp transforms/wavelet/convolution.cpp transforms/wavelet/wt.cpp
textures/gabor.cpp textures/tamura.cpp textures/haralick/CVIPtexture.cpp textures/haralick/haralick.cpp
textures/zernike/zernike.cpp textures/zernike/complex.cpp
statistics/CombFirst4Moments.cpp statistics/FeatureStatistics.cpp colors/FuzzyCalc.cpp gsl/specfunc.cpp
wndchrm_src/TrainingSet.cpp wndchrm_src/signatures.cpp wndchrm_src/WORMfile.cpp"
OBJS=""
pids=""
for f in $FILES; do
  o="$OUT/obj/$(echo "$f" | tr '/' '_' | sed 's/\.cpp$/.o/')"
  OBJS="$OBJS $o"
  if [ ! -f "$o" ] || [ "$SRC/$f" -nt "$o" ]; then
    $CXX $FLAGS -c "$SRC/$f" -o "$o" &
    pids="$pids $!"
  fi
done
for f in fftw_shim.cpp tiff_stub.cpp ref_capi.cpp; do
  o="$OUT/obj/shim_${f%.cpp}.o"
  OBJS="$OBJS $o"
  $CXX $FLAGS -ffp-contract=off -c "$HERE/ref_shim/$f" -o "$o" &
  pids="$pids $!"
done
for p in $pids; do wait "$p"; done
$CXX -shared -o "$OUT/libwndref.so" $OBJS
echo "built $OUT/libwndref.so"
