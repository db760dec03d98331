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
//   ref_cpu joblist   LIST OUT  scriptFileRead(LIST); OUT: one JSON line per job with the
//                     arguments HilbertTransform received and the globals it would read
//   ref_cpu bmp       BMP OUT   bmp_header + read_bmp; OUT: i32 nr, nc; u8 image[nr nc]
//   ref_cpu phimap    IN OUT    IN: i32 status, sx, sy; f64 angle x, y; f32 phase[sx sy],
//                               amp[sx sy]; outputImg writes OUT
//   ref_cpu check     IN OUT    IN: i32 n; f32 limitSTD, limitRange; f32 v[n]; OUT: i32 checkArray
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
int scriptFileRead(char *script);
void bmp_header(char *filename, int &nr, int &nc);
void read_bmp(char *filename, int nr, int nc, unsigned char *image);
struct microImg {
    float phase;
    float amp;
};
void outputImg(char *fpath, microImg *output, bool status, double angleX, double angleY, int sizeX, int sizeY);
bool checkArray(float *array2D, float limitSTD, float limitRange, int size);
// the job globals scriptFileRead fills (defined with the reference's initial values in ref_cpu.cpp)
extern int rowSize, colSize, ReconFlag, ReconSave, SizeType, ResizeFlag, SavePhaseStack, SaveAmpStack;
extern double Nmed, Mag, CameraPixelSize, wavelength, criteriaRange, criteriaSTD;

static FILE *g_jobs;

static void json_str(FILE *o, const char *k, const char *v)
{
    fprintf(o, "\"%s\": \"", k);
    for (const char *c = v; *c; c++) {
        if (*c == '"' || *c == '\\') fputc('\\', o);
        if ((unsigned char)*c < 0x20) fprintf(o, "\\u%04x", (unsigned char)*c);
        else fputc(*c, o);
    }
    fputs("\", ", o);
}

// Stands in for the job itself: records what scriptFileRead passed and set.
void HilbertTransform(char *SPDir, char *BGDir, char *AngDir, char *SaveDir, int rowPts[], int colPts[], int rowSize,
                      int colSize, int StartNo, int SpaceNo, int EndNo)
{
    if (!g_jobs) return;
    fputc('{', g_jobs);
    json_str(g_jobs, "sp_dir", SPDir);
    json_str(g_jobs, "bg_dir", BGDir);
    json_str(g_jobs, "ang_dir", AngDir);
    json_str(g_jobs, "save_dir", SaveDir);
    fprintf(g_jobs,
            "\"row_pts\": [%d, %d], \"col_pts\": [%d, %d], \"row_size\": %d, \"col_size\": %d, "
            "\"start_no\": %d, \"space_no\": %d, \"end_no\": %d, \"recon_flag\": %d, \"recon_save\": %d, "
            "\"size_type\": %d, \"resize_flag\": %d, \"n_med\": %.17g, \"mag\": %.17g, "
            "\"camera_pixel_um\": %.17g, \"wavelength_nm\": %.17g, \"save_phase_stack\": %d, "
            "\"save_amp_stack\": %d, \"criteria_range\": %.17g, \"criteria_std\": %.17g}\n",
            rowPts[0], rowPts[1], colPts[0], colPts[1], rowSize, colSize, StartNo, SpaceNo, EndNo, ReconFlag,
            ReconSave, SizeType, ResizeFlag, Nmed, Mag, CameraPixelSize, wavelength, SavePhaseStack, SaveAmpStack,
            criteriaRange, criteriaSTD);
}

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
        fprintf(stderr, "usage: ref_cpu floodfill|bilinear|fft2d|fft3d|shift3d|joblist|bmp|phimap|check IN OUT\n");
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
    } else if (!strcmp(op, "joblist")) {
        g_jobs = fopen(argv[3], "w");
        if (!g_jobs) return fclose(f), 2;
        const int ok = scriptFileRead(argv[2]);
        fclose(g_jobs);
        g_jobs = nullptr;
        rc = ok == 1 ? 0 : 3;
    } else if (!strcmp(op, "bmp")) {
        int nr = 0, nc = 0;
        bmp_header(argv[2], nr, nc);
        if (!sane((long)nr * nc) || nr <= 0 || nc <= 0) return fclose(f), 2;
        std::vector<unsigned char> img((size_t)nr * nc);
        read_bmp(argv[2], nr, nc, img.data());
        const int32_t d[2] = {nr, nc};
        FILE *o = fopen(argv[3], "wb");
        if (!o) return fclose(f), 2;
        const bool ok = fwrite(d, sizeof d, 1, o) == 1 && fwrite(img.data(), 1, img.size(), o) == img.size();
        rc = fclose(o) == 0 && ok ? 0 : 2;
    } else if (!strcmp(op, "phimap")) {
        int32_t d[3];
        double ang[2];
        r.get(d, 3);
        r.get(ang, 2);
        const long n = (long)d[1] * d[2];
        if (!r.ok || !sane(n)) return fclose(f), 2;
        std::vector<float> ph(n), am(n);
        r.get(ph.data(), n);
        r.get(am.data(), n);
        if (!r.ok) return fclose(f), 2;
        std::vector<microImg> img(n);
        for (long i = 0; i < n; i++) img[i] = {ph[i], am[i]};
        outputImg(argv[3], img.data(), d[0] != 0, ang[0], ang[1], d[1], d[2]);
    } else if (!strcmp(op, "check")) {
        int32_t n;
        float lim[2];
        r.get(&n, 1);
        r.get(lim, 2);
        if (!r.ok || !sane(n)) return fclose(f), 2;
        std::vector<float> v(n);
        r.get(v.data(), n);
        if (!r.ok) return fclose(f), 2;
        const int32_t out = checkArray(v.data(), lim[0], lim[1], n) ? 1 : 0;
        rc = put(argv[3], &out, sizeof out) ? 0 : 2;
    } else {
        fprintf(stderr, "unknown operation %s\n", op);
        rc = 2;
    }
    fclose(f);
    return rc;
}
