#!/bin/sh
# Build recipe for oracle/_ref/libref_cpu.so: the reference's OWN CPU code,
# compiled from the reference sources where they lie, used only to pin the
# oracle restatement (tests/golden/gen_golden.py).  Nothing is copied into the
# repository: the extracted snippets and the .so live under oracle/_ref/,
# which git ignores.
#
#   test/cl_unittest.cc:138-166  cpu_aos_asta / cpu_soa_asta (macro T)
#   test/unittest.cu:68-82        templated cpu_aos_asta
#   include/plan.hpp              Transposition::Next / GetNumCycles, Factorize
#
# plan.hpp's GPUInfo queries an OpenCL context; no OpenCL headers exist here,
# so a 12-line type stub is supplied.  The stubbed queries are never reached
# (Transposition is built with a NULL context, plan.hpp:27-30 then uses its
# defaults), so only the reference's integer arithmetic is exercised.
#
# Usage: sh oracle/build_ref.sh [reference-root]
# The root is the argument, else $LM_REFERENCE, else the checkout's place in
# the build container (/root/reference); where none exists the recipe exits
# with status 2 and builds nothing.
set -e
REF=${1:-${LM_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/test/cl_unittest.cc" ] || [ ! -f "$REF/include/plan.hpp" ]; then
  echo "build_ref.sh: reference not found at $REF" >&2
  exit 2
fi
mkdir -p "$OUT"

sed -n '138,166p' "$REF/test/cl_unittest.cc" > "$OUT/cl_cpu_layouts.inc"
sed -n '68,82p' "$REF/test/unittest.cu" > "$OUT/cu_cpu_aos_asta.inc"
# Refuse to build if the line ranges no longer hold the expected functions.
head -1 "$OUT/cl_cpu_layouts.inc" | grep -q '^void cpu_aos_asta(T \*src' || { echo "unexpected cl_unittest.cc:138" >&2; exit 3; }
grep -q '^void cpu_soa_asta(T \*src' "$OUT/cl_cpu_layouts.inc" || { echo "unexpected cl_unittest.cc:153" >&2; exit 3; }
head -1 "$OUT/cu_cpu_aos_asta.inc" | grep -q '^template <class T>' || { echo "unexpected unittest.cu:68" >&2; exit 3; }

cat > "$OUT/ref_shim.cc" <<'EOF'
// Generated by oracle/build_ref.sh -- wraps reference code for ctypes.
#include <cassert>
#include <cstdint>
#include <cstdlib>
#include <cstddef>
#include <string>
#include <vector>
typedef struct _cl_context *cl_context;
typedef struct _cl_device_id *cl_device_id;
typedef int cl_int;
typedef unsigned long cl_ulong;
#define CL_SUCCESS 0
#define CL_CONTEXT_DEVICES 0x1081
#define CL_DEVICE_LOCAL_MEM_SIZE 0x1023
#define CL_DEVICE_MAX_WORK_GROUP_SIZE 0x1004
static inline cl_int clGetContextInfo(cl_context, int, size_t, void *, size_t *) { return -1; }
static inline cl_int clGetDeviceInfo(cl_device_id, int, size_t, void *, size_t *) { return -1; }
#include "plan.hpp"

namespace ref_u8 { typedef uint8_t T;
#include "cl_cpu_layouts.inc"
}
namespace ref_u16 { typedef uint16_t T;
#include "cl_cpu_layouts.inc"
}
namespace ref_u32 { typedef uint32_t T;
#include "cl_cpu_layouts.inc"
}
namespace ref_u64 { typedef uint64_t T;
#include "cl_cpu_layouts.inc"
}
namespace ref_cu {
#include "cu_cpu_aos_asta.inc"
}

#define LM_REF_EXPORT(TY, NS, SUF)                                                   \
  extern "C" void ref_cl_aos_asta_##SUF(void *s, void *d, int h, int w, int t) {     \
    NS::cpu_aos_asta((TY *)s, (TY *)d, h, w, t);                                     \
  }                                                                                  \
  extern "C" void ref_cl_soa_asta_##SUF(void *s, void *d, int h, int w, int t) {     \
    NS::cpu_soa_asta((TY *)s, (TY *)d, h, w, t);                                     \
  }                                                                                  \
  extern "C" void ref_cu_aos_asta_##SUF(void *s, void *d, int h, int w, int t) {     \
    ref_cu::cpu_aos_asta<TY>((TY *)s, (TY *)d, h, w, t);                             \
  }
LM_REF_EXPORT(uint8_t, ref_u8, u8)
LM_REF_EXPORT(uint16_t, ref_u16, u16)
LM_REF_EXPORT(uint32_t, ref_u32, u32)
LM_REF_EXPORT(uint64_t, ref_u64, u64)

extern "C" unsigned ref_next(unsigned i, int m, int n) {
  Transposition t(m, n);
  return t.Next(i);
}
extern "C" long long ref_num_cycles(int m, int n) {
  Transposition t(m, n);
  return (long long)t.GetNumCycles();
}
extern "C" int ref_tile_options(int n, int *out, int cap) {
  Factorize f(n);
  f.tiling_options();
  std::vector<int> &v = f.get_tile_sizes();
  for (size_t i = 0; i < v.size() && (int)i < cap; i++) out[i] = v[i];
  return (int)v.size();
}
extern "C" int ref_factors(int n, int *primes, int *exps, int cap) {
  Factorize f(n);
  int k = 0;
  for (std::map<int, int>::const_iterator it = f.get_factors().begin();
       it != f.get_factors().end(); ++it, ++k)
    if (k < cap) { primes[k] = it->first; exps[k] = it->second; }
  return k;
}
EOF
g++ -O2 -fPIC -shared -w -I"$OUT" -I"$REF/include" "$OUT/ref_shim.cc" -o "$OUT/libref_cpu.so"
echo "built $OUT/libref_cpu.so"
