"""Assembles the reference's own CUDA pipeline sources for the comparison build.

COMPARISON INFRASTRUCTURE ONLY (like the rest of oracle/): nothing in the product
links or runs it.  The reference (y-h-Lin/cTDM) builds as one Visual Studio project
whose driver file cTDM/HilbertTransform.cu does not compile outside Windows, so the
comparison build takes:

* whole files, unmodified: cTDM/FFT.cu (cuFFT wrappers and shift / scale kernels),
  cTDM/Recon_kernel.cu (median, Ewald mapping, F/F2, est_n, modify, check),
  cTDM/DCT_Unwrapping.cu, cTDM/FastUnwrapping.cu (driven by harness_fast.cu) and the
  headers they include;
* five functions cut verbatim from cTDM/HilbertTransform.cu by line range:
  extractQPI_AlgorithmA (:1546-1585), obtainRadius (:3425-3455), get1stOrder_new
  (:3566-3586), calcWrapPhase (:3618-3639) and bilinear_interpolation_kernel
  (:3658-3723), behind a prologue that declares the file-scope globals they use
  (defined by oracle/refcuda/harness.cu, which drives them in the order of the
  reference's job loop and BatchRecon);
* for QPI Algorithm B (the reference's default QPI_Method = 0), a second unit qpi_b.cu:
  extractQPI_AlgorithmB (:1587-1606), sequence1DFFT (:1608-1662), real2cufft
  (:1664-1702), copySharedMem (:1704-1726), HistogramFT (:1728-1748), shiftArray
  (:1750-1763), CropFTdomain (:1811-1823), calcWrapPhase and
  bilinear_interpolation_kernel, driven by oracle/refcuda/harness_b.cu;
* for the Goldstein residues, gold_res.cu: cudaPhaseResidues (cTDM/Goldstein.cu:52-103) and
  cudaMod (:1193-1201), driven by oracle/refcuda/harness_res.cu.

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
         "dct8x8_kernel2.cuh", "Common.h", "FastUnwrapping.cu", "FastUnwrapping.cuh"]

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


CUTS_B = [
    (1587, 1606, "void extractQPI_AlgorithmB("),
    (1608, 1662, "void sequence1DFFT("),
    (1664, 1702, "__global__ void real2cufft("),
    (1704, 1726, "__global__ void copySharedMem("),
    (1728, 1748, "__global__ void HistogramFT("),
    (1750, 1763, "__global__ void shiftArray("),
    (1811, 1823, "__global__ void CropFTdomain("),
    (3618, 3639, "__global__ void calcWrapPhase("),
    (3658, 3723, "__global__ void bilinear_interpolation_kernel("),
]

PROLOGUE_B = """// Cut from cTDM/HilbertTransform.cu by oracle/refcuda/assemble.py (comparison build only).
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <time.h>
#include <cufft.h>
#include <thrust/device_ptr.h>
#include <thrust/extrema.h>
const int TILE_DIM = 32;
const int BLOCK_ROWS = 32;
extern int blocksInX, blocksInY, blocksInX2, blocksInY2, blocksInX3, blocksInY3, blocksInX4, blocksInY4;
extern int Nx2, Ny2;
extern int max_idx_seq1D;
extern float *cuSP_PE_temp, *cuBG_PE_temp, *cuSP_PE_resample, *cuBG_PE_resample;
extern cufftComplex *device_PE_FFT, *out_PE_FFT;
extern float *sumFFT_PE_1D;
extern cufftHandle plan_1D_C2C_FORWARD_FT, plan_1D_C2C_INVERSE_FT;
extern clock_t s_datatransfer, e_datatransfer, s_wrap, e_wrap;
extern float dataTransfer_time, wrap_time;
void sequence1DFFT(float *ResampleArray, cufftComplex *out_array, int Nx, int Ny, int frame);
__global__ void real2cufft(cufftComplex *odata, const float *idata);
__global__ void copySharedMem(cufftComplex *odata, const cufftComplex *idata, const float scale);
__global__ void HistogramFT(float *sumFFT_1D, cufftComplex *device_FFT, int Nx, int Ny);
__global__ void shiftArray(cufftComplex *device_FFT, int Nx, int Ny);
__global__ void CropFTdomain(cufftComplex *device_FFT, cufftComplex *device_crop, int Nx, int Ny, int center);
__global__ void bilinear_interpolation_kernel(float *__restrict__ d_result_1, const float *__restrict__ d_data_1,
                                              float *__restrict__ d_result_2, const float *__restrict__ d_data_2,
                                              const int M1, const int N1, const int M2, const int N2);
"""


# Goldstein residues: cudaPhaseResidues (cTDM/Goldstein.cu:52-103) and the cudaMod it calls
# (:1193-1201), driven by harness_res.cu.
CUTS_RES = [
    (52, 103, "__global__ void cudaPhaseResidues("),
    (1193, 1201, "__device__ float cudaMod("),
]

PROLOGUE_RES = """// Cut from cTDM/Goldstein.cu by oracle/refcuda/assemble.py (comparison build only).
#define _USE_MATH_DEFINES
#include <math.h>
#include <cuda_runtime.h>
__device__ float cudaMod(float a, float b);
"""


def cut(lines, cuts, prologue, name="HilbertTransform.cu"):
    parts = [prologue]
    for first, last, head in cuts:
        chunk = lines[first - 1:last]
        if not chunk or not chunk[0].startswith(head) or not chunk[-1].startswith("}"):
            raise SystemExit(f"{name}:{first}-{last} is not {head}... (reference changed?)")
        parts.append(f"// cTDM/{name}:{first}-{last}\n" + "\n".join(chunk) + "\n")
    return "\n".join(parts)


def main(root):
    src = os.path.join(root, "cTDM")
    os.makedirs(OUT, exist_ok=True)
    for name in WHOLE:
        shutil.copyfile(os.path.join(src, name), os.path.join(OUT, name))
    lines = open(os.path.join(src, "HilbertTransform.cu"), encoding="latin-1").read().split("\n")
    lines = [ln.rstrip("\r") for ln in lines]
    with open(os.path.join(OUT, "qpi_a.cu"), "w", encoding="latin-1") as f:
        f.write(cut(lines, CUTS, PROLOGUE))
    with open(os.path.join(OUT, "qpi_b.cu"), "w", encoding="latin-1") as f:
        f.write(cut(lines, CUTS_B, PROLOGUE_B))
    # Goldstein.cu carries BIG5 comments: latin-1 keeps the bytes
    glines = [ln.rstrip("\r") for ln in open(os.path.join(src, "Goldstein.cu"), encoding="latin-1").read().split("\n")]
    with open(os.path.join(OUT, "gold_res.cu"), "w", encoding="latin-1") as f:
        f.write(cut(glines, CUTS_RES, PROLOGUE_RES, "Goldstein.cu"))
    return OUT


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/refcuda/assemble.py <reference root (the y-h-Lin/cTDM checkout)>")
    print(main(sys.argv[1]))
