// Runs one of the reference's host functions (cut into oracle/_ref/refcpu/src/ref_cpu.cpp
// by oracle/refcpu/assemble.py) on a little-endian binary input file and writes its
// output array.  COMPARISON INFRASTRUCTURE ONLY: tests run it in a child process with
// a time limit, because FloodFill spins forever on inputs whose sweeps stall.
//
//   ref_cpu floodfill IN OUT  IN: i32 w, h; f32 cut[w h]; f32 phi[w h]   OUT: f32 unwrapped[w h]
//   ref_cpu bilinear  IN OUT  IN: i32 m1, n1, m2, n2; f32 img[n1 m1]     OUT: f32 [n2 m2]
//   ref_cpu fft2d     IN OUT  IN: i32 nx, ny, dir; c64 [nx ny]           OUT: c64 [nx ny]
//   ref_cpu fft3d     IN OUT  IN: i32 nx, ny, nz, dir; c64 [nx ny nz]    OUT: c64 [nx ny nz]
//   ref_cpu shift3d   IN OUT  IN: i32 w, h, s; c64 [w h s]               OUT: c64 [w h s]
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

void FloodFill(float *BranchCut, int sizeX, int sizeY, float *phi, float *IMUnwrapped, float *IMMask);
void bilinear(float *input, float *output, int M1, int N1, int M2, int N2);
int FFT2D(std::complex<float> *c, int nx, int ny, int dir);
void FFT3D(std::complex<float> *c, int nx, int ny, int nz, int dir);
void FFT3Dshift(std::complex<float> *input, int width, int height, int slice);

namespace {

struct Reader {
    FILE *f;
    bool ok = true;
    template <class T>
    void get(T *dst, size_t n)
    {
        if (ok && fread(dst, sizeof(T), n, f) != n) ok = false;
    }
};

bool put(const char *path, const void *p, size_t bytes)
{
    FILE *f = fopen(path, "wb");
    if (!f) return false;
    const bool ok = fwrite(p, 1, bytes, f) == bytes;
    return fclose(f) == 0 && ok;
}

bool sane(long n) { return n > 0 && n <= (1L << 28); }

}  // namespace

int main(int argc, char **argv)
{
    if (argc != 4) {
        fprintf(stderr, "usage: ref_cpu floodfill|bilinear|fft2d|fft3d|shift3d IN OUT\n");
        return 2;
    }
    const char *op = argv[1];
    FILE *f = fopen(argv[2], "rb");
    if (!f) {
        fprintf(stderr, "cannot open %s\n", argv[2]);
        return 2;
    }
    Reader r{f};
    int rc = 0;
    if (!strcmp(op, "floodfill")) {
        int32_t d[2];
        r.get(d, 2);
        const long n = (long)d[0] * d[1];
        if (!r.ok || !sane(n)) return fclose(f), 2;
        std::vector<float> cut(n), phi(n), out(n, 0.f), mask(n, 1.f);
        r.get(cut.data(), n);
        r.get(phi.data(), n);
        if (!r.ok) return fclose(f), 2;
        FloodFill(cut.data(), d[0], d[1], phi.data(), out.data(), mask.data());
        rc = put(argv[3], out.data(), n * sizeof(float)) ? 0 : 2;
    } else if (!strcmp(op, "bilinear")) {
        int32_t d[4];
        r.get(d, 4);
        const long n1 = (long)d[0] * d[1], n2 = (long)d[2] * d[3];
        if (!r.ok || !sane(n1) || !sane(n2)) return fclose(f), 2;
        std::vector<float> in(n1), out(n2);
        r.get(in.data(), n1);
        if (!r.ok) return fclose(f), 2;
        bilinear(in.data(), out.data(), d[0], d[1], d[2], d[3]);
        rc = put(argv[3], out.data(), n2 * sizeof(float)) ? 0 : 2;
    } else if (!strcmp(op, "fft2d") || !strcmp(op, "fft3d") || !strcmp(op, "shift3d")) {
        const bool two = !strcmp(op, "fft2d"), shift = !strcmp(op, "shift3d");
        int32_t d[4] = {1, 1, 1, 0};
        r.get(d, two || shift ? 3 : 4);
        if (two) {
            d[3] = d[2];
            d[2] = 1;
        }
        const long n = (long)d[0] * d[1] * d[2];
        if (!r.ok || !sane(n)) return fclose(f), 2;
        std::vector<std::complex<float>> c(n);
        r.get(c.data(), n);
        if (!r.ok) return fclose(f), 2;
        if (two) {
            if (!FFT2D(c.data(), d[0], d[1], d[3])) rc = 3;
        } else if (shift) {
            FFT3Dshift(c.data(), d[0], d[1], d[2]);
        } else {
            FFT3D(c.data(), d[0], d[1], d[2], d[3]);
        }
        if (rc == 0) rc = put(argv[3], c.data(), n * sizeof(c[0])) ? 0 : 2;
    } else {
        fprintf(stderr, "unknown operation %s\n", op);
        rc = 2;
    }
    fclose(f);
    return rc;
}
