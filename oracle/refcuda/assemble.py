"""Assembles the reference's own CUDA pipeline sources for the comparison build.

COMPARISON INFRASTRUCTURE ONLY (like the rest of oracle/): nothing in the product
links or runs it.  The reference (y-h-Lin/cTDM) builds as one Visual Studio project
whose driver file cTDM/HilbertTransform.cu does not compile outside Windows, so the
comparison build takes:

* whole files, unmodified: cTDM/FFT.cu (cuFFT wrappers and shift / scale kernels),
  cTDM/Recon_kernel.cu (median, Ewald mapping, F/F2, est_n, modify, check),
  cTDM/DCT_Unwrapping.cu and the headers they include;
* five functions cut verbatim from cTDM/HilbertTransform.cu by line range:
  extractQPI_AlgorithmA (:1546-1585), obtainRadius (:3425-3455), get1stOrder_new
  (:3566-3586), calcWrapPhase (:3618-3639) and bilinear_interpolation_kernel
  (:3658-3723), behind a prologue that declares the file-scope globals they use
  (defined by oracle/refcuda/harness.cu, which drives them in the order of the
  reference's job loop and BatchRecon).

Output: oracle/_ref/refcuda/src/ (git-ignored; it travels with the tree to the GPU
machine, where oracle/refcuda/Makefile builds it with nvcc and cuFFT).

Usage: python oracle/refcuda/assemble.py <reference root (the y-h-Lin/cTDM checkout)>
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref", "refcuda", "src")

WHOLE = ["FFT.cu", "FFT.cuh", "Recon_kernel.cu", "Recon_kernel.cuh", "DCT_Unwrapping.cu", "DCT_Unwrapping.cuh",
         "dct8x8_kernel2.cuh", "Common.h"]

# (first line, last line, text the first line must start with), 1-based inclusive
CUTS = [
    (1546, 1585, "void extractQPI_AlgorithmA("),
    (3425, 3455, "void obtainRadius("),
    (3566, 3586, "__global__ void get1stOrder_new("),
    (3618, 3639, "__global__ void calcWrapPhase("),
    (3658, 3723, "__global__ void bilinear_interpolation_kernel("),
]

PROLOGUE = """// Cut from cTDM/HilbertTransform.cu by oracle/refcuda/assemble.py (comparison build only).
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <time.h>
#include <cufft.h>
#include "FFT.cuh"
extern int blocksInX, blocksInY, blocksInX2, blocksInY2, blocksInX3, blocksInY3, blocksInX4, blocksInY4;
extern int Nx2, Ny2;
extern int rCircle, cCircle, radiusCircle;
extern cufftComplex *cuSP, *cuBG, *cuSP2, *cuBG2;
extern cufftHandle plan_2D_C2C_FORWARD_s1, plan_2D_C2C_INVERSE_s2;
extern clock_t s_datatransfer, e_datatransfer, s_wrap, e_wrap;
extern float dataTransfer_time, wrap_time;
void obtainRadius(cufftComplex *, int &, int &, int &, int, int);
__global__ void get1stOrder_new(cufftComplex *out, cufftComplex *in, int radius, int r, int c, int sizeX, int sizeY);
"""


def main(root):
    src = os.path.join(root, "cTDM")
    os.makedirs(OUT, exist_ok=True)
    for name in WHOLE:
        shutil.copyfile(os.path.join(src, name), os.path.join(OUT, name))
    lines = open(os.path.join(src, "HilbertTransform.cu"), encoding="latin-1").read().split("\n")
    parts = [PROLOGUE]
    for first, last, head in CUTS:
        chunk = lines[first - 1:last]
        if not chunk or not chunk[0].startswith(head) or not chunk[-1].startswith("}"):
            raise SystemExit(f"HilbertTransform.cu:{first}-{last} is not {head}... (reference changed?)")
        parts.append(f"// cTDM/HilbertTransform.cu:{first}-{last}\n" + "\n".join(chunk) + "\n")
    with open(os.path.join(OUT, "qpi_a.cu"), "w", encoding="latin-1") as f:
        f.write("\n".join(parts))
    return OUT


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/refcuda/assemble.py <reference root (the y-h-Lin/cTDM checkout)>")
    print(main(sys.argv[1]))
