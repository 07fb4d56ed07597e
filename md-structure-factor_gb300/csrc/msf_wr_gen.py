"""Writes msf_wr.cuh: w_R^k = exp(-2 pi i k / R) for the composite radices of
the mixed-radix register FFT, cos/sin in FP64 (exact 0 and +-1 on the axes)
rounded to float.  Run: python msf_wr_gen.py > msf_wr.cuh"""
import math
import struct

RADICES = [6, 9, 10, 12, 15, 18, 20, 25, 27]


def lit(x):
    v = struct.unpack("f", struct.pack("f", float(x)))[0]
    if v == 0.0:
        return "-0.0f" if math.copysign(1.0, v) < 0 else "0.0f"
    s = "%.9g" % v
    if "e" not in s and "." not in s:
        s += ".0"
    return s + "f"


def cos_sin(k, r):
    if k == 0:
        return 1.0, 0.0
    if 4 * k == r:
        return 0.0, 1.0
    if 2 * k == r:
        return -1.0, 0.0
    if 4 * k == 3 * r:
        return 0.0, -1.0
    a = 2.0 * math.pi * k / r
    return math.cos(a), math.sin(a)


def main():
    out = [
        "// msf_wr.cuh -- w_R^k = exp(-2 pi i k / R), k < R, for the composite in-register",
        "// radices of the mixed-radix FFT (msf_mixed.cuh): cos and sin of 2 pi k / R",
        "// evaluated in FP64 and rounded to float, written out as literals by",
        "// msf_wr_gen.py.  Every index is a compile-time constant once the DFT loops",
        "// unroll, so these fold into immediates.",
        "#pragma once",
        "",
        "#include <cuda_runtime.h>",
        "",
        "namespace msf {",
        "namespace mixed {",
        "",
        "template <int R> struct WR;",
        "",
    ]
    for r in RADICES:
        out += [f"template <> struct WR<{r}> {{",
                "  static __host__ __device__ constexpr float2 w(int k) {",
                f"    switch (k % {r}) {{"]
        for k in range(r):
            c, s = cos_sin(k, r)
            out.append(f"      case {k}: return make_float2({lit(c)}, {lit(-s)});")
        out += ["    }", "    return make_float2(1.0f, 0.0f);", "  }", "};", ""]
    out += ["}  // namespace mixed", "}  // namespace msf"]
    print("\n".join(out))


if __name__ == "__main__":
    main()
