"""The drop-in boundary as a reference build sees it: a C++ translation unit that
includes include/ctdm.h and then declares the reference's own prototypes, as its
headers write them, inside extern "C" (with cufftComplex as ctdm_cfloat), compiles
and links against libctdm_gb300.so.  A C function declared twice with a different
return or parameter type is a compile error, so any drift between the library's
signatures and the reference's fails here.  The program then calls the one
host-only entry (checkArray) and takes the address of every other one, so the
link resolves each symbol; no GPU is needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Prototypes as the reference declares them (file:line within cTDM/).
REFERENCE_PROTOTYPES = r"""
/* Recon_kernel.cuh:31 */
void MedianFilter(float *PhaseData, float *AmpData, float *Phase_img, float *Amp_img, int nx, int ny, int nz);
/* Recon_kernel.cuh:37 */
void CopyDataArray(cufftComplex *u_sp, float *phase, float *amp, int sizeX, int sizeY, int sizeZ, int numZ);
/* Recon_kernel.cuh:41 */
void EdwardSphere(cufftComplex *u_sp, cufftComplex *F, float * C, float fm0, float df, float AngX, float AngY
	, int sizeX, int sizeY, int sizeZ);
/* Recon_kernel.cuh:51 */
void initial_F_and_F2(float *C, cufftComplex *cuF, cufftComplex *cuF2, float recon_dx , int Image_Width, int Image_Height, int Image_Slice);
/* Recon_kernel.cuh:56 */
void est_n_3D(cufftComplex *n, cufftComplex *F, float recon_k2, float recon_med
					, int Image_Width, int Image_Height, int Image_Slice);
/* Recon_kernel.cuh:63 */
void modify_F_3D(cufftComplex *n, cufftComplex *F, float recon_k2, float recon_med
					, int Image_Width, int Image_Height, int Image_Slice);
/* Recon_kernel.cuh:70 */
void check_F_3D(cufftComplex *F, cufftComplex *F2, int Image_Width, int Image_Height, int Image_Slice);
/* FFT.cuh:25 */
void cuFFT2D(cufftComplex *ImgArray, int sizeX, int sizeY, int dir);
/* FFT.cuh:29 */
void cuFFT3D(cufftComplex *ImgArray, int sizeX, int sizeY, int sizeZ, int dir);
/* DCT_Unwrapping.cuh:106 */
void DCT_UWLS_Unwrapped(float *ImgDst, float *ImgSrc, int sizeX, int sizeY);
/* FastUnwrapping.cuh:12 */
void FastUnwrapping(float *ImgSrc, float *ImgDst, int sizeX, int sizeY);
/* Goldstein.cuh:41 */
void cudaGoldsteinUnwrap2D(float *cu_phi, float *cu_UnWrapPhase, int sizeX, int sizeY,int frameNumber);
/* HilbertTransform.cuh:120 */
int scriptFileRead(char *);
/* HilbertTransform.cuh:127 */
void HilbertTransform(char *,char *,char *,char *,int rowPts[], int colPts[],int,int,int,int,int);
/* HilbertTransform.cuh:132 */
void BatchRecon(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY, int ReconFrame);
/* HilbertTransform.cuh:133 */
void BatchReconPOCS(float *PhaseStack, float *AmpStack, float *sampleAngleRadX, float *sampleAngleRadY, int ReconFrame);
/* HilbertTransform.cuh:155 */
float AngCal_GPU(float *src, int sizeX, int sizeY, int frame, int totalFrame);
/* HilbertTransform.cuh:158 */
bool checkArray(float *array2D, float limitSTD, float limitRange, int size);
/* HilbertTransform.cuh:170 */
void extractQPI_AlgorithmA(cufftComplex *SP, cufftComplex *BG, cufftComplex *cuSP_FFT, cufftComplex *cuBG_FFT, int Nx, int Ny, int frame);
/* HilbertTransform.cuh:171 */
void extractQPI_AlgorithmB(float *SP, float *BG, cufftComplex *cuSP_FFT, cufftComplex *cuBG_FFT, int Nx, int Ny, int frame);
"""

NAMES = ["MedianFilter", "CopyDataArray", "EdwardSphere", "initial_F_and_F2", "est_n_3D", "modify_F_3D",
         "check_F_3D", "cuFFT2D", "cuFFT3D", "DCT_UWLS_Unwrapped", "FastUnwrapping", "cudaGoldsteinUnwrap2D",
         "scriptFileRead", "HilbertTransform", "BatchRecon", "BatchReconPOCS", "AngCal_GPU", "checkArray",
         "extractQPI_AlgorithmA", "extractQPI_AlgorithmB"]

PROGRAM = r"""
#include <cstdio>
#include "ctdm.h"
typedef ctdm_cfloat cufftComplex;
extern "C" {
%(protos)s
}
int main()
{
    const void *entries[] = {%(addrs)s};
    for (const void *p : entries)
        if (!p) return 3;
    float v[4] = {0.f, 0.f, 0.f, 4.f};
    const bool a = checkArray(v, 1.0f, 100.0f, 4);   /* std sqrt(3) > 1 */
    const bool b = checkArray(v, 2.0f, 100.0f, 4);
    const bool c = checkArray(v, 2.0f, 3.5f, 4);     /* range 4 > 3.5 */
    std::printf("%%d %%d %%d\n", (int)a, (int)b, (int)c);
    return (a && !b && c) ? 0 : 2;
}
"""


def _program():
    addrs = ", ".join(f"(const void *)&{n}" for n in NAMES)
    return PROGRAM % {"protos": REFERENCE_PROTOTYPES, "addrs": addrs}


def test_every_reference_prototype_is_declared():
    for n in NAMES:
        assert f" {n}(" in REFERENCE_PROTOTYPES


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_reference_prototypes_compile_link_and_run(tmp_path):
    from ctdm_gb300 import build
    so = build.build()
    src = tmp_path / "ref_boundary.cpp"
    src.write_text(_program())
    exe = tmp_path / "ref_boundary"
    libdir = os.path.dirname(so)
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lctdm_gb300", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath-link,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.split() == ["1", "0", "1"]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_a_changed_signature_is_caught(tmp_path):
    """The check itself: a prototype whose return type differs from the library's
    (checkArray returning int) does not compile."""
    src = tmp_path / "drift.cpp"
    src.write_text('#include "ctdm.h"\nextern "C" { int checkArray(float *, float, float, int); }\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode != 0
