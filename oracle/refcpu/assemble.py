"""Assembles the reference's own host (CPU) functions of the path for the CPU comparison build.

COMPARISON INFRASTRUCTURE ONLY (like the rest of oracle/): nothing in the product links
or runs it.  The functions are cut verbatim, by line range, from the y-h-Lin/cTDM
checkout; their files do not compile as a whole outside Windows / without CUDA, the
functions themselves are plain C++:

* cTDM/Goldstein.cu: FloodFill (:643-1095) and sumAdjoin (:1097-1105), the serial
  flood fill of Goldstein unwrapping;
* cTDM/HilbertTransform.cu: bilinear (:2404-2435), the host resize; scriptFileRead
  (:70-175) and obtainParameter (:200-221), the job list and parameter-file reading
  (the driver supplies a HilbertTransform that records the job instead of running it);
  outputImg (:2437-2455), the .phimap writer; bmp_header (:2680-2692) and read_bmp
  (:2694-2731), the frame reader; checkArray (:3056-3092), the frame check;
* cTDM/FFT.cu: FFT (:29-103), Powerof2 (:352-372), FFT2D (:380-434), FFT3D
  (:436-543) and FFT3Dshift (:272-296), the host transforms and octant swap.

A prologue supplies what their files' headers did (the standard headers, CUDA's int2,
`using namespace std`, the microImg pair, the job globals scriptFileRead fills with the
reference's initial values, cTDM/HilbertTransform.cu:10-40) and maps MSVC's strtok_s
to POSIX strtok_r (the same arguments and meaning).  Output: oracle/_ref/refcpu/src/ref_cpu.cpp (git-ignored);
oracle/refcpu/Makefile compiles it with g++ together with oracle/refcpu/driver.cpp.

Usage: python oracle/refcpu/assemble.py <reference root (the y-h-Lin/cTDM checkout)>
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref", "refcpu", "src")

# (file, first line, last line, text the first line must start with), 1-based inclusive
CUTS = [
    ("FFT.cu", 29, 103, "int FFT(int dir,int m,double *x,double *y)"),
    ("FFT.cu", 272, 296, "void FFT3Dshift(complex<float> *input"),
    ("FFT.cu", 352, 372, "int Powerof2(int n, int *m, int *twopm)"),
    ("FFT.cu", 380, 434, "int FFT2D(complex<float> *c, int nx, int ny, int dir)"),
    ("FFT.cu", 436, 543, "void FFT3D(complex<float> *c, int nx, int ny, int nz, int dir)"),
    ("Goldstein.cu", 643, 1095, "void FloodFill(float *BranchCut,int sizeX, int sizeY"),
    ("Goldstein.cu", 1097, 1105, "int sumAdjoin(float *Adjoin,int rowSize,int colSize)"),
    ("HilbertTransform.cu", 2404, 2435, "void bilinear(float *input, float *output"),
    ("HilbertTransform.cu", 70, 175, "int scriptFileRead(char* script)"),
    ("HilbertTransform.cu", 200, 221, "char *obtainParameter(char *strLine)"),
    ("HilbertTransform.cu", 2437, 2455, "void outputImg(char *fpath, microImg *output"),
    ("HilbertTransform.cu", 2680, 2692, "void bmp_header(char *filename, int &nr, int &nc)"),
    ("HilbertTransform.cu", 2694, 2731, "void read_bmp(char *filename, int nr, int nc, unsigned char *image)"),
    ("HilbertTransform.cu", 3056, 3092, "bool checkArray(float *array2D, float limitSTD, float limitRange, int size)"),
]

PROLOGUE = """// Cut from the y-h-Lin/cTDM sources by oracle/refcpu/assemble.py (comparison build only).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <iostream>
using namespace std;
struct int2 { int x, y; };
int FFT(int, int, double *, double *);
int Powerof2(int, int *, int *);
int FFT2D(complex<float> *, int, int, int);
int sumAdjoin(float *Adjoin, int rowSize, int colSize);
#include <cstring>
#define strtok_s strtok_r
typedef struct microImg { float phase; float amp; } microImg;
char *SPDir = (char *)malloc(256), *BGDir = (char *)malloc(256), *AngDir = (char *)malloc(256),
     *SaveDir = (char *)malloc(256);
int rowSize = 1024, colSize = 1024;
int ReconFlag = 1, ReconSave = 0, SizeType = 0, ResizeFlag = 1, SavePhaseStack = 0, SaveAmpStack = 0;
double Nmed = 1.333, Mag = 85.0, CameraPixelSize = 5.5, wavelength = 532, criteriaRange = 3 * M_PI,
       criteriaSTD = 0.5;
char *obtainParameter(char *strLine);
void HilbertTransform(char *SPDir, char *BGDir, char *AngDir, char *SaveDir, int rowPts[], int colPts[],
                      int rowSize, int colSize, int StartNo, int SpaceNo, int EndNo);
"""


def main(root):
    src = os.path.join(root, "cTDM")
    os.makedirs(OUT, exist_ok=True)
    parts = [PROLOGUE]
    cache = {}
    for name, first, last, head in CUTS:
        if name not in cache:
            # Goldstein.cu carries BIG5 comments and one BIG5 string: latin-1 keeps the bytes
            cache[name] = open(os.path.join(src, name), encoding="latin-1").read().split("\n")
        chunk = [ln.rstrip("\r") for ln in cache[name][first - 1:last]]
        if not chunk or not chunk[0].startswith(head) or not chunk[-1].startswith("}"):
            raise SystemExit(f"{name}:{first}-{last} is not {head}... (reference changed?)")
        parts.append(f"// cTDM/{name}:{first}-{last}\n" + "\n".join(chunk) + "\n")
    with open(os.path.join(OUT, "ref_cpu.cpp"), "w", encoding="latin-1") as f:
        f.write("\n".join(parts))
    return OUT


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/refcpu/assemble.py <reference root (the y-h-Lin/cTDM checkout)>")
    print(main(sys.argv[1]))
