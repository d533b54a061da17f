"""Generates sg_dft.cuh: fully unrolled in-register complex DFTs of size
2..32 (forward e^{-2 pi i jk/P} and backward e^{+2 pi i jk/P}, unnormalised).

Each DFT is an iterative radix-2 decimation-in-time network on a register
array loaded in bit-reversed order; the twiddles are emitted as literals so
that every butterfly constant-folds (trivial +-1, +-i twiddles cost no
multiply).  Run:  python gen_dft.py > sg_dft.cuh   (a build step; the output
is committed).
"""
import math

SIZES = [2, 4, 8, 16, 32]


def bitrev(i, bits):
    r = 0
    for b in range(bits):
        if i & (1 << b):
            r |= 1 << (bits - 1 - b)
    return r


def emit(P, inverse):
    bits = P.bit_length() - 1
    name = "sg_dft%d_%s" % (P, "bwd" if inverse else "fwd")
    out = []
    out.append("template <typename T>")
    out.append("__device__ __forceinline__ void %s(cplx<T> (&a)[%d]) {" % (name, P))
    # bit reversal permutation as register renaming
    out.append("  cplx<T> b[%d];" % P)
    for i in range(P):
        out.append("  b[%d] = a[%d];" % (i, bitrev(i, bits)))
    length = 2
    while length <= P:
        half = length // 2
        for start in range(0, P, length):
            for j in range(half):
                u, v = start + j, start + j + half
                ang = 2.0 * math.pi * j / length
                c, s = math.cos(ang), (math.sin(ang) if inverse else -math.sin(ang))
                if j == 0:
                    out.append("  { cplx<T> t = b[%d]; b[%d] = b[%d] - t; b[%d] = b[%d] + t; }"
                               % (v, v, u, u, u))
                elif 4 * j == length:
                    # multiply by -i (forward) or +i (backward)
                    if inverse:
                        out.append("  { cplx<T> t = cplx<T>{-b[%d].y, b[%d].x}; b[%d] = b[%d] - t; b[%d] = b[%d] + t; }"
                                   % (v, v, v, u, u, u))
                    else:
                        out.append("  { cplx<T> t = cplx<T>{b[%d].y, -b[%d].x}; b[%d] = b[%d] - t; b[%d] = b[%d] + t; }"
                                   % (v, v, v, u, u, u))
                else:
                    out.append("  { cplx<T> t = cmul(b[%d], cplx<T>{T(%r), T(%r)}); b[%d] = b[%d] - t; b[%d] = b[%d] + t; }"
                               % (v, c, s, v, u, u, u))
        length *= 2
    for i in range(P):
        out.append("  a[%d] = b[%d];" % (i, i))
    out.append("}")
    return "\n".join(out)


def main():
    print("// Generated by gen_dft.py -- do not edit.")
    print("// In-register unnormalised DFTs of size 2..32 (radix-2 DIT, literal twiddles).")
    print("#pragma once")
    print('#include "sg_cplx.cuh"')
    print()
    for P in SIZES:
        for inv in (False, True):
            print(emit(P, inv))
            print()
    print("template <int P, bool INV, typename T> struct SgDft;")
    for P in SIZES:
        for inv in (False, True):
            print("template <typename T> struct SgDft<%d, %s, T> { __device__ __forceinline__ static void run(cplx<T> (&a)[%d]) { sg_dft%d_%s(a); } };"
                  % (P, "true" if inv else "false", P, P, "bwd" if inv else "fwd"))


if __name__ == "__main__":
    main()
