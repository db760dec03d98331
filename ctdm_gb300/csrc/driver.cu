// JobList-driven driver and the reference's on-disk formats (y-h-Lin/cTDM
// scriptFileRead / HilbertTransform, cTDM/HilbertTransform.cu:70-175, 327-1230).
//
// A job file lists parameter files; each parameter file holds 20 "key=value" fields
// in a fixed order (:96-120): SPDir, BGDir, AngDir, SaveDir, rowPts[0..1],
// colPts[0..1], ReconFlag, ReconSave, SizeType, ResizeFlag, Nmed, Mag,
// CameraPixelSize (um), wavelength (nm), SavePhaseStack, SaveAmpStack,
// criteriaRange, criteriaSTD.  Two optional trailing keys set what the reference
// fixes at compile time: QPI_Method (reference numbering, default 0 = Algorithm B)
// and IterTime (default 100).
//
// A job (ReconFlag 0 or 1) reads frames SPDir/Buffer<k>.bmp and BGDir/Buffer<k>.bmp
// (8-bit grey, read_bmp's transposed storage), estimates each frame's illumination
// angle from AngDir (X/ and Y/ sub-folders, else AngDir/Buffer<k>.bmp; AngCal_GPU),
// retrieves phase and amplitude (QPI Algorithm B or A), DCT-unwraps, resizes the maps
// to the hologram size, checks each frame (checkArray), and writes
// SaveDir/buffer%03d.phimap per frame (plus Phase/Amp raw files on request).
// ReconFlag 1 stacks the centre R x R windows (Combine2Stack, ResizeFlag 1) and
// ReconFlag 2 reloads them from the .phimap files (LoadDateFromDir); the frames that
// passed the check (RefreshStack) go through BatchRecon, which writes
// 3D-RI-{Complex,Real,Imag}_RxRxR.rimap.  Frames are processed as one batch on the
// GPU.  Paths use '/'; the reference's '\' separators are Windows paths.
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "kernels_front.cuh"

using namespace ctdm;

namespace {

constexpr int kBmpHeader = 54, kBmpPalette = 1024;

std::string join(const std::string &dir, const std::string &name)
{
    std::string s = dir.empty() ? std::string(".") : dir;
    if (s.back() != '/') s += '/';
    return s + name;
}

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// count_file_num (:2479-2530, its Linux branch): entries of `dir` whose name contains
// `head`, hidden entries skipped.
int count_files(const std::string &dir, const char *head)
{
    DIR *d = opendir(dir.c_str());
    if (!d) return 0;
    int n = 0;
    while (dirent *e = readdir(d)) {
        if (e->d_name[0] == '.') continue;
        if (strstr(e->d_name, head)) n++;
    }
    closedir(d);
    return n;
}

// checkArray (:3056-3092): the frame fails when the standard deviation (double
// accumulation, population variance) exceeds limit_std or the float range exceeds
// limit_range.
bool check_array(const float *v, long n, float limit_std, float limit_range)
{
    double mean = 0;
    float mx = -99999.0f, mn = 99999.0f;
    for (long i = 0; i < n; i++) {
        mean += v[i];
        if (v[i] > mx) mx = v[i];
        if (v[i] < mn) mn = v[i];
    }
    mean /= n;
    double var = 0;
    for (long i = 0; i < n; i++) var += (v[i] - mean) * (v[i] - mean);
    var /= n;
    return std::sqrt(var) > limit_std || (float)std::fabs(mx - mn) > limit_range;
}

// The reference's job defaults (cTDM/HilbertTransform.cu:11-35).
ctdm_job_file default_job()
{
    ctdm_job_file j;
    memset(&j, 0, sizeof j);
    strcpy(j.sp_dir, ".");
    strcpy(j.bg_dir, ".");
    strcpy(j.ang_dir, ".");
    strcpy(j.save_dir, ".");
    j.row_pts[1] = j.col_pts[1] = 1023;
    j.recon_flag = 1;
    j.resize_flag = 1;
    j.n_med = 1.333;
    j.mag = 85.0;
    j.camera_pixel_um = 5.5;
    j.wavelength_nm = 532.0;
    j.criteria_range = 3 * CTDM_PI_D;
    j.criteria_std = 0.5;
    j.qpi_method = CTDM_QPI_B;
    j.iter_time = 100;
    return j;
}

ctdm_job_file g_job = default_job();   // the job scriptFileRead parsed last (the reference's globals)

struct KV {
    std::string key, value;
};

// Every "key=value" of a parameter file in order, the way scriptFileRead reads them
// (:96-120): fscanf("%*[^=]%s") skips to the next '=' and takes the white-space free
// token from there, and obtainParameter (:200-221) keeps the last non-empty piece of
// that token split at '=' ("=a=b" gives "b").  Spaces after '=' are skipped here, where
// the reference would read a token of '=' alone and return an unset pointer.  The key
// is the last word before '='.
std::vector<KV> key_values(const std::string &text)
{
    std::vector<KV> out;
    size_t pos = 0;
    while (true) {
        const size_t eq = text.find('=', pos);
        if (eq == std::string::npos) break;
        size_t ke = eq;
        while (ke > pos && isspace((unsigned char)text[ke - 1])) ke--;
        size_t kb = ke;
        while (kb > pos && !isspace((unsigned char)text[kb - 1])) kb--;
        size_t b = eq + 1;
        while (b < text.size() && (text[b] == ' ' || text[b] == '\t')) b++;
        size_t e = b;
        while (e < text.size() && !isspace((unsigned char)text[e])) e++;
        // the last non-empty '='-separated piece of [b, e)
        size_t ve = e;
        while (ve > b && text[ve - 1] == '=') ve--;
        size_t vb = ve;
        while (vb > b && text[vb - 1] != '=') vb--;
        out.push_back({text.substr(kb, ke - kb), text.substr(vb, ve - vb)});
        pos = e;
    }
    return out;
}

bool same_key(const std::string &a, const char *b)
{
    if (a.size() != strlen(b)) return false;
    for (size_t i = 0; i < a.size(); i++)
        if (tolower((unsigned char)a[i]) != tolower((unsigned char)b[i])) return false;
    return true;
}

bool set_path(char *dst, const std::string &v)
{
    if (v.size() >= 256) return false;
    std::string p = v;
    for (char &ch : p)
        if (ch == '\\') ch = '/';   // the reference's Windows separators
    strcpy(dst, p.c_str());
    return true;
}

// ---- frame-level pieces of HilbertTransform's loop
// read_bmp storage (image[c * N + r], r the row from the top) as float: the layout the
// reference hands to Algorithm B (SP_float_All, :655-660).
void storage_to_float(const uint8_t *img, long n, float *out)
{
    for (long i = 0; i < n; i++) out[i] = (float)img[i];
}

// The transposed, row-major image (x fastest) the reference hands to Algorithm A and to
// AngCal_GPU (SP_cu_All / AngImgX, :709-718).
void storage_to_image(const uint8_t *img, int N, float *out)
{
    for (int j = 0; j < N; j++)
        for (int i = 0; i < N; i++) out[i + (long)j * N] = (float)img[j + (long)i * N];
}

// Host bilinear N1 -> N2 (bilinear, :2404-2435), float arithmetic as written.
void bilinear(const float *in, float *out, int M1, int N1, int M2, int N2)
{
    const float xr = ((float)(M1 - 1)) / M2, yr = ((float)(N1 - 1)) / N2;
    long o = 0;
    for (int i = 0; i < N2; i++)
        for (int j = 0; j < M2; j++) {
            const int x = (int)(xr * j), y = (int)(yr * i);
            const float xd = (xr * j) - x, yd = (yr * i) - y;
            const long idx = (long)y * M1 + x;
            const float A = in[idx], B = in[idx + 1], C = in[idx + M1], D = in[idx + M1 + 1];
            out[o++] = (float)(A * (1 - xd) * (1 - yd) + B * (xd) * (1 - yd) + C * (yd) * (1 - xd) + D * (xd * yd));
        }
}

// Combine2Stack (:1316-1430): frame `f` of the R x R stacks from an N x N map, NaN/inf
// scrubbed (phase -> 0, amplitude -> 1).  ResizeFlag 1 takes the centred window,
// ResizeFlag 0 the bilinear resize.
void combine_to_stack(const float *ph, const float *am, int N, int R, int resize_flag, float *ph_stack,
                      float *am_stack, int f)
{
    const long rr = (long)R * R;
    float *P = ph_stack + f * rr, *A = am_stack + f * rr;
    if (N == R) {
        memcpy(P, ph, sizeof(float) * rr);
        memcpy(A, am, sizeof(float) * rr);
    } else if (resize_flag == 0) {
        bilinear(ph, P, N, N, R, R);
        bilinear(am, A, N, N, R, R);
    } else {
        const int o = (N - R) / 2;
        for (int j = 0; j < R; j++)
            for (int i = 0; i < R; i++) {
                P[i + (long)R * j] = ph[(i + o) + (long)N * (j + o)];
                A[i + (long)R * j] = am[(i + o) + (long)N * (j + o)];
            }
    }
    for (long i = 0; i < rr; i++) {
        if (std::isnan(P[i]) || std::isinf(P[i])) P[i] = 0.f;
        if (std::isnan(A[i]) || std::isinf(A[i])) A[i] = 1.f;
    }
}

// RefreshStack (:1487-1544): keeps the frames whose status is set, in order.
int refresh_stack(std::vector<float> &ph, std::vector<float> &am, const std::vector<int> &status,
                  std::vector<float> &angx, std::vector<float> &angy, long rr)
{
    int k = 0;
    for (size_t z = 0; z < status.size(); z++) {
        if (!status[z]) continue;
        if ((int)z != k) {
            memmove(ph.data() + k * rr, ph.data() + z * rr, sizeof(float) * rr);
            memmove(am.data() + k * rr, am.data() + z * rr, sizeof(float) * rr);
            angx[k] = angx[z];
            angy[k] = angy[z];
        }
        k++;
    }
    ph.resize(k * rr);
    am.resize(k * rr);
    angx.resize(k);
    angy.resize(k);
    return k;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    template <class T>
    T *as() { return static_cast<T *>(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes); }
};

// The illumination angle of AngCal_GPU from the flat index of the spectrum peak.
float angle_of_peak(long peak, int N, double n_med, double wavelength_nm, double mag, double pixel_um)
{
    const int posX = (int)(peak % N);
    const float fm = (float)(n_med / (wavelength_nm * 1e-9));
    const float fx = (float)((N / 2 - 1 - posX) * 1 / (N * pixel_um * 1e-6));
    const float st = (float)mag * fx / fm;
    return st < 0 ? std::fabs(std::asin(st)) : -std::fabs(std::asin(st));
}

// Peak of one host angle image through device scratch (img: N*N floats, spec: N*N
// complex, key: one 64-bit word).
ctdm_status peak_of_image(const float *h_img, int N, float *img, float2 *spec, unsigned long long *key, long *peak)
{
    cudaError_t e = cudaMemcpy(img, h_img, sizeof(float) * N * N, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = angcal_peak(img, N, spec, key, 0);
    unsigned long long k = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&k, key, sizeof k, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail_cuda(e, "angle estimation");
    *peak = (long)(~(unsigned)(k & 0xffffffffull));
    return CTDM_OK;
}

bool angle_size_ok(int N) { return N >= 16 && N <= 2048 && (N & (N - 1)) == 0; }

}  // namespace

// ---------------------------------------------------------------- formats
extern "C" ctdm_status ctdm_read_bmp(const char *path, int *width, int *height, uint8_t *image)
{
    if (!path || !width || !height) return fail_invalid("ctdm_read_bmp: NULL argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail_io(std::string("cannot open ") + path);
    unsigned char hdr[kBmpHeader];
    if (fread(hdr, 1, kBmpHeader, fp) != (size_t)kBmpHeader || hdr[0] != 'B' || hdr[1] != 'M') {
        fclose(fp);
        return fail_io(std::string("not a BMP file: ") + path);
    }
    int nr, nc;
    memcpy(&nr, hdr + 18, 4);   // bmp_header (:2680-2692): width, then height
    memcpy(&nc, hdr + 22, 4);
    const int bpp = hdr[28] | (hdr[29] << 8);
    *width = nr;
    *height = nc;
    if (!image) {
        fclose(fp);
        clear_error();
        return CTDM_OK;
    }
    if (bpp != 8 || nr <= 0 || nc <= 0) {
        fclose(fp);
        return fail_invalid("ctdm_read_bmp: 8-bit grey images only");
    }
    // read_bmp (:2694-2731): skip header and palette, rows bottom-up padded to 4 bytes,
    // stored transposed (image[j * nr + i])
    fseek(fp, kBmpHeader + kBmpPalette, SEEK_SET);
    int linewidth = nc;
    if (linewidth & 3) linewidth = (linewidth | 3) + 1;
    std::vector<unsigned char> line(linewidth);
    for (int i = nr - 1; i >= 0; i--) {
        if (fread(line.data(), 1, linewidth, fp) != (size_t)linewidth) {
            fclose(fp);
            return fail_io(std::string("truncated BMP: ") + path);
        }
        for (int j = 0; j < nc; j++) image[(long)j * nr + i] = line[j];
    }
    fclose(fp);
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_write_phimap(const char *path, int status, double angle_x, double angle_y, int size_x,
                                         int size_y, const float *phase, const float *amp)
{
    if (!path || !phase || !amp || size_x < 1 || size_y < 1) return fail_invalid("ctdm_write_phimap: bad argument");
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail_io(std::string("cannot write ") + path);
    // outputImg (:2437-2455): bool, two doubles, two ints, then (phase, amp) pairs
    const unsigned char st = status ? 1 : 0;
    bool ok = fwrite(&st, 1, 1, fp) == 1 && fwrite(&angle_x, 8, 1, fp) == 1 && fwrite(&angle_y, 8, 1, fp) == 1 &&
              fwrite(&size_x, 4, 1, fp) == 1 && fwrite(&size_y, 4, 1, fp) == 1;
    const long n = (long)size_x * size_y;
    std::vector<float> pairs(2 * n);
    for (long i = 0; i < n; i++) {
        pairs[2 * i] = phase[i];
        pairs[2 * i + 1] = amp[i];
    }
    ok = ok && fwrite(pairs.data(), sizeof(float), 2 * n, fp) == (size_t)(2 * n);
    fclose(fp);
    if (!ok) return fail_io(std::string("short write: ") + path);
    clear_error();
    return CTDM_OK;
}

extern "C" ctdm_status ctdm_read_phimap(const char *path, int *status, double *angle_x, double *angle_y, int *size_x,
                                        int *size_y, float *phase, float *amp)
{
    if (!path || !size_x || !size_y) return fail_invalid("ctdm_read_phimap: NULL argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail_io(std::string("cannot open ") + path);
    unsigned char st = 0;
    double ax = 0, ay = 0;
    int sx = 0, sy = 0;
    bool ok = fread(&st, 1, 1, fp) == 1 && fread(&ax, 8, 1, fp) == 1 && fread(&ay, 8, 1, fp) == 1 &&
              fread(&sx, 4, 1, fp) == 1 && fread(&sy, 4, 1, fp) == 1;
    if (!ok || sx < 1 || sy < 1) {
        fclose(fp);
        return fail_io(std::string("bad .phimap header: ") + path);
    }
    if (status) *status = st ? 1 : 0;
    if (angle_x) *angle_x = ax;
    if (angle_y) *angle_y = ay;
    *size_x = sx;
    *size_y = sy;
    if (phase || amp) {
        const long n = (long)sx * sy;
        std::vector<float> pairs(2 * n);
        if (fread(pairs.data(), sizeof(float), 2 * n, fp) != (size_t)(2 * n)) {
            fclose(fp);
            return fail_io(std::string("truncated .phimap: ") + path);
        }
        for (long i = 0; i < n; i++) {
            if (phase) phase[i] = pairs[2 * i];
            if (amp) amp[i] = pairs[2 * i + 1];
        }
    }
    fclose(fp);
    clear_error();
    return CTDM_OK;
}

namespace ctdm {
ctdm_status write_ri_volume(const std::string &dir, int R, int save_mode, const ctdm_cfloat *h_ri, const char *ext)
{
    if (!h_ri || R < 1 || save_mode < 0 || save_mode > 2) return fail_invalid("RI volume export: bad argument");
    // export (:2013-2041): complex64, or the real / imaginary part as float32
    char name[96];
    const char *kind = save_mode == 0 ? "Complex" : (save_mode == 1 ? "Real" : "Imag");
    snprintf(name, sizeof name, "3D-RI-%s_%dx%dx%d.%s", kind, R, R, R, ext);
    const std::string path = join(dir, name);
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return fail_io("cannot write " + path);
    const long n = (long)R * R * R;
    bool ok;
    if (save_mode == 0) {
        ok = fwrite(h_ri, sizeof(ctdm_cfloat), n, fp) == (size_t)n;
    } else {
        std::vector<float> part(n);
        for (long i = 0; i < n; i++) part[i] = save_mode == 1 ? h_ri[i].x : h_ri[i].y;
        ok = fwrite(part.data(), sizeof(float), n, fp) == (size_t)n;
    }
    fclose(fp);
    if (!ok) return fail_io("short write: " + path);
    clear_error();
    return CTDM_OK;
}
}  // namespace ctdm

extern "C" ctdm_status ctdm_write_rimap(const char *dir, int R, int save_mode, const ctdm_cfloat *h_ri)
{
    return write_ri_volume(dir ? dir : ".", R, save_mode, h_ri, "rimap");
}

extern "C" int ctdm_check_frame(const float *phase, int N, int resize_flag, double limit_std, double limit_range)
{
    if (!phase || N < 4) return 1;
    if (resize_flag == 0) return check_array(phase, (long)N * N, 0.5, 5 * CTDM_PI_D) ? 1 : 0;
    // the centre half of the map (:1107-1117)
    std::vector<float> area((size_t)(N / 2) * (N / 2));
    for (int j = N / 4; j < N * 3 / 4; j++)
        for (int i = N / 4; i < N * 3 / 4; i++) area[(i - N / 4) + (long)(j - N / 4) * (N / 2)] = phase[i + (long)j * N];
    return check_array(area.data(), (long)area.size(), limit_std, limit_range) ? 1 : 0;
}

extern "C" ctdm_status ctdm_angle_from_image(const float *h_img, int N, double n_med, double wavelength_nm, double mag,
                                             double camera_pixel_um, float *angle, long *peak)
{
    if (!h_img || !angle) return fail_invalid("ctdm_angle_from_image: NULL argument");
    if (!angle_size_ok(N)) return fail_invalid("ctdm_angle_from_image: N must be a power of two in 16..2048");
    if (!(n_med > 0) || !(wavelength_nm > 0) || !(camera_pixel_um > 0))
        return fail_invalid("ctdm_angle_from_image: optics must be positive");
    DevBuf img, spec, key;
    cudaError_t e = img.alloc(sizeof(float) * N * N);
    if (e == cudaSuccess) e = spec.alloc(sizeof(float2) * N * N);
    if (e == cudaSuccess) e = key.alloc(sizeof(unsigned long long));
    if (e != cudaSuccess) return fail_cuda(e, "ctdm_angle_from_image alloc");
    long pk = 0;
    ctdm_status st = peak_of_image(h_img, N, img.as<float>(), spec.as<float2>(), key.as<unsigned long long>(), &pk);
    if (st != CTDM_OK) return st;
    *angle = angle_of_peak(pk, N, n_med, wavelength_nm, mag, camera_pixel_um);
    if (peak) *peak = pk;
    clear_error();
    return CTDM_OK;
}

// ---------------------------------------------------------------- job files
extern "C" void ctdm_job_defaults(ctdm_job_file *job)
{
    if (job) *job = default_job();
}

extern "C" ctdm_status ctdm_parse_job_file(const char *path, ctdm_job_file *job)
{
    if (!path || !job) return fail_invalid("ctdm_parse_job_file: NULL argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail_io(std::string("cannot open parameter file ") + path);
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, n);
    fclose(fp);
    const std::vector<KV> kv = key_values(text);
    if (kv.size() < 20)
        return fail_io(std::string("parameter file ") + path + " has " + std::to_string(kv.size()) +
                       " key=value fields, 20 needed");
    ctdm_job_file j = default_job();
    // the 20 fields in the order scriptFileRead reads them (:96-120); names are not checked
    if (!set_path(j.sp_dir, kv[0].value) || !set_path(j.bg_dir, kv[1].value) || !set_path(j.ang_dir, kv[2].value) ||
        !set_path(j.save_dir, kv[3].value))
        return fail_invalid("ctdm_parse_job_file: a folder path is 256 characters or longer");
    j.row_pts[0] = atoi(kv[4].value.c_str());
    j.row_pts[1] = atoi(kv[5].value.c_str());
    j.col_pts[0] = atoi(kv[6].value.c_str());
    j.col_pts[1] = atoi(kv[7].value.c_str());
    j.recon_flag = atoi(kv[8].value.c_str());
    j.recon_save = atoi(kv[9].value.c_str());
    j.size_type = atoi(kv[10].value.c_str());
    j.resize_flag = atoi(kv[11].value.c_str());
    j.n_med = atof(kv[12].value.c_str());
    j.mag = atof(kv[13].value.c_str());
    j.camera_pixel_um = atof(kv[14].value.c_str());
    j.wavelength_nm = atof(kv[15].value.c_str());
    j.save_phase_stack = (int)atof(kv[16].value.c_str());
    j.save_amp_stack = (int)atof(kv[17].value.c_str());
    j.criteria_range = atof(kv[18].value.c_str());
    j.criteria_std = atof(kv[19].value.c_str());
    for (size_t i = 20; i < kv.size(); i++) {
        if (same_key(kv[i].key, "QPI_Method")) j.qpi_method = atoi(kv[i].value.c_str());
        else if (same_key(kv[i].key, "IterTime")) j.iter_time = atoi(kv[i].value.c_str());
        else return fail_invalid(("ctdm_parse_job_file: unknown key " + kv[i].key).c_str());
    }
    *job = j;
    clear_error();
    return CTDM_OK;
}

// ---------------------------------------------------------------- the job
namespace {

ctdm_status check_job(const ctdm_job_file &j)
{
    if (j.recon_flag < 0 || j.recon_flag > 2) return fail_invalid("job: ReconFlag must be 0, 1 or 2");
    if (j.recon_save < 0 || j.recon_save > 2) return fail_invalid("job: ReconSave must be 0, 1 or 2");
    if (j.size_type < 0 || j.size_type > 1) return fail_invalid("job: SizeType must be 0 or 1");
    if (j.resize_flag < 0 || j.resize_flag > 1) return fail_invalid("job: ResizeFlag must be 0 or 1");
    if (j.qpi_method == 2)
        return fail_invalid("job: QPI_Method 2 (full-size circular window with a fitted radius) is not built");
    if (j.qpi_method != CTDM_QPI_B && j.qpi_method != CTDM_QPI_A) return fail_invalid("job: QPI_Method must be 0 or 1");
    if (j.iter_time < 0 || j.iter_time > 100000) return fail_invalid("job: IterTime outside 0..100000");
    if (!(j.n_med > 0) || !(j.mag > 0) || !(j.camera_pixel_um > 0) || !(j.wavelength_nm > 0))
        return fail_invalid("job: Nmed, Mag, CameraPixelSize and wavelength must be positive");
    return CTDM_OK;
}

struct Stacks {
    std::vector<float> ph, am, angx, angy;
    std::vector<int> status;
};

ctdm_status read_frame(const std::string &path, int N, std::vector<uint8_t> &img)
{
    int w = 0, h = 0;
    ctdm_status st = ctdm_read_bmp(path.c_str(), &w, &h, nullptr);
    if (st != CTDM_OK) return st;
    if (w != N || h != N) return fail_invalid(("Wrong size: " + path + " is not " + std::to_string(N) + " x " +
                                               std::to_string(N)).c_str());
    return ctdm_read_bmp(path.c_str(), &w, &h, img.data());
}

bool write_raw(const std::string &path, const float *v, long n)
{
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) return false;
    const bool ok = fwrite(v, sizeof(float), n, fp) == (size_t)n;
    fclose(fp);
    return ok;
}

// Frames 1..F from the SP / BG / angle folders (HilbertTransform, ReconFlag 0 and 1).
ctdm_status process_frames(const ctdm_job_file &jb, int R, ctdm_job_result &r, Stacks &S)
{
    const int F = std::min(count_files(jb.sp_dir, "Buffer"), count_files(jb.bg_dir, "Buffer"));
    if (F < 1) return fail_io(std::string("no Buffer*.bmp frames in ") + jb.sp_dir + " and " + jb.bg_dir);
    int nrSP, ncSP, nrBG, ncBG;
    ctdm_status st = ctdm_read_bmp(join(jb.sp_dir, "Buffer1.bmp").c_str(), &nrSP, &ncSP, nullptr);
    if (st == CTDM_OK) st = ctdm_read_bmp(join(jb.bg_dir, "Buffer1.bmp").c_str(), &nrBG, &ncBG, nullptr);
    if (st != CTDM_OK) return st;
    if (nrSP != nrBG || ncSP != ncBG) return fail_invalid("Wrong size! (sample and background frames differ)");
    const int N = nrSP;
    if (ncSP != N || N < 64 || N > 2048 || (N & (N - 1)))
        return fail_invalid("job: holograms must be square with a power-of-two side in 64..2048");
    if (jb.recon_flag == 1 && jb.resize_flag == 1 && N < R)
        return fail_invalid("job: ResizeFlag 1 crops an R x R window, so the holograms must be at least R wide");
    mkdir(jb.save_dir, 0755);
    if (!is_dir(jb.save_dir)) return fail_io(std::string("cannot create ") + jb.save_dir);
    r.frames = F;
    r.n_holo = N;
    const int M = N / 4;
    const long nn = (long)N * N, mm = (long)M * M, rr = (long)R * R;
    const bool xy = is_dir(join(jb.ang_dir, "X")) && is_dir(join(jb.ang_dir, "Y"));
    const bool alg_b = jb.qpi_method == CTDM_QPI_B;
    // frames per batch: 256 MiB of sample holograms on the device, or CTDM_JOB_BATCH_FRAMES
    int C = std::max(1, std::min({F, (int)((1l << 28) / (4 * nn)), max_angles()}));
    if (const char *env = getenv("CTDM_JOB_BATCH_FRAMES"))
        if (atoi(env) > 0) C = std::min(C, atoi(env));

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
    ctdm_ctx *ctx = nullptr;
    st = ctdm_ctx_create(dev, &ctx);
    if (st != CTDM_OK) return st;
    struct CtxGuard {
        ctdm_ctx *c;
        ~CtxGuard() { ctdm_ctx_destroy(c); }
    } guard{ctx};
    DevBuf d_holo, d_bg, d_ph, d_am, d_unw, d_phN, d_amN, d_ang, d_spec, d_key;
    if ((e = d_holo.alloc(sizeof(float) * C * nn)) != cudaSuccess || (e = d_bg.alloc(sizeof(float) * C * nn)) != cudaSuccess ||
        (e = d_ph.alloc(sizeof(float) * C * mm)) != cudaSuccess || (e = d_am.alloc(sizeof(float) * C * mm)) != cudaSuccess ||
        (e = d_unw.alloc(sizeof(float) * C * mm)) != cudaSuccess ||
        (e = d_phN.alloc(sizeof(float) * C * nn)) != cudaSuccess ||
        (e = d_amN.alloc(sizeof(float) * C * nn)) != cudaSuccess || (e = d_ang.alloc(sizeof(float) * nn)) != cudaSuccess ||
        (e = d_spec.alloc(sizeof(float2) * nn)) != cudaSuccess ||
        (e = d_key.alloc(sizeof(unsigned long long))) != cudaSuccess)
        return fail_cuda(e, "job device buffers");
    std::vector<uint8_t> img(nn);
    std::vector<float> h_holo(C * nn), h_bg(C * nn), h_ang(nn), h_ph(C * nn), h_am(C * nn);
    S.status.assign(F, 1);
    S.angx.assign(F, 0.f);
    S.angy.assign(F, 0.f);
    if (jb.recon_flag == 1) {
        S.ph.assign((size_t)F * rr, 0.f);
        S.am.assign((size_t)F * rr, 0.f);
    }
    int center2[2] = {-1, -1}, carrier3[3] = {-1, -1, -1};
    char name[64];
    for (int s0 = 0; s0 < F; s0 += C) {
        const int n = std::min(C, F - s0);
        for (int f = 0; f < n; f++) {
            const int k = s0 + f + 1;   // frame number, from 1
            snprintf(name, sizeof name, "Buffer%d.bmp", k);
            if ((st = read_frame(join(jb.sp_dir, name), N, img)) != CTDM_OK) return st;
            if (alg_b) storage_to_float(img.data(), nn, h_holo.data() + f * nn);
            else storage_to_image(img.data(), N, h_holo.data() + f * nn);
            if ((st = read_frame(join(jb.bg_dir, name), N, img)) != CTDM_OK) return st;
            if (alg_b) storage_to_float(img.data(), nn, h_bg.data() + f * nn);
            else storage_to_image(img.data(), N, h_bg.data() + f * nn);
            // angles (AngCal_GPU on the X image, and on the Y image when X/ and Y/ exist)
            long pk = 0;
            const std::string ax = xy ? join(join(jb.ang_dir, "X"), name) : join(jb.ang_dir, name);
            if ((st = read_frame(ax, N, img)) != CTDM_OK) return st;
            storage_to_image(img.data(), N, h_ang.data());
            st = peak_of_image(h_ang.data(), N, d_ang.as<float>(), d_spec.as<float2>(),
                               d_key.as<unsigned long long>(), &pk);
            if (st != CTDM_OK) return st;
            S.angx[k - 1] = angle_of_peak(pk, N, jb.n_med, jb.wavelength_nm, jb.mag, jb.camera_pixel_um);
            if (xy) {
                if ((st = read_frame(join(join(jb.ang_dir, "Y"), name), N, img)) != CTDM_OK) return st;
                storage_to_image(img.data(), N, h_ang.data());
                st = peak_of_image(h_ang.data(), N, d_ang.as<float>(), d_spec.as<float2>(),
                                   d_key.as<unsigned long long>(), &pk);
                if (st != CTDM_OK) return st;
                S.angy[k - 1] = angle_of_peak(pk, N, jb.n_med, jb.wavelength_nm, jb.mag, jb.camera_pixel_um);
            }
        }
        if ((e = cudaMemcpy(d_holo.p, h_holo.data(), sizeof(float) * n * nn, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(d_bg.p, h_bg.data(), sizeof(float) * n * nn, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail_cuda(e, "job upload");
        // QPI with one background per frame; frame 1 fixes the carrier for the later frames
        if (alg_b) {
            st = ctdm_qpi_b(ctx, N, n, d_holo.as<float>(), d_bg.as<float>(), 1, center2, d_ph.as<float>(),
                            d_am.as<float>(), nullptr);
            center2[1] = center2[0];   // frames after the first take the background's column
        } else {
            st = ctdm_qpi(ctx, N, M, n, d_holo.as<float>(), d_bg.as<float>(), 1, carrier3, d_ph.as<float>(),
                          d_am.as<float>(), nullptr);
        }
        if (st == CTDM_OK) st = ctdm_unwrap_dct(ctx, n, M, CTDM_UNWRAP_REF, d_ph.as<float>(), d_unw.as<float>(), nullptr);
        if (st != CTDM_OK) return st;
        e = resize_maps(d_unw.as<float>(), d_am.as<float>(), n, M, N, d_phN.as<float>(), d_amN.as<float>(), 0);
        if (e == cudaSuccess) e = cudaMemcpy(h_ph.data(), d_phN.p, sizeof(float) * n * nn, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(h_am.data(), d_amN.p, sizeof(float) * n * nn, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail_cuda(e, "job maps");
        for (int f = 0; f < n; f++) {
            const int k = s0 + f + 1;
            const float *ph = h_ph.data() + f * nn, *am = h_am.data() + f * nn;
            const int ok = ctdm_check_frame(ph, N, jb.resize_flag, jb.criteria_std, jb.criteria_range) ? 0 : 1;
            S.status[k - 1] = ok;
            if (!ok) r.rejected++;
            snprintf(name, sizeof name, "buffer%03d.phimap", k);
            st = ctdm_write_phimap(join(jb.save_dir, name).c_str(), ok, S.angx[k - 1], S.angy[k - 1], N, N, ph, am);
            if (st != CTDM_OK) return st;
            if (jb.recon_flag == 1)
                combine_to_stack(ph, am, N, R, jb.resize_flag, S.ph.data(), S.am.data(), k - 1);
            if (jb.save_phase_stack == 1) {
                snprintf(name, sizeof name, "Phase%03d_%dx%d.raw", k, N, N);
                if (!write_raw(join(jb.save_dir, name), ph, nn)) return fail_io("cannot write " + join(jb.save_dir, name));
            }
            if (jb.save_amp_stack == 1) {
                snprintf(name, sizeof name, "Amp%03d_%dx%d.raw", k, N, N);
                if (!write_raw(join(jb.save_dir, name), am, nn)) return fail_io("cannot write " + join(jb.save_dir, name));
            }
        }
    }
    return CTDM_OK;
}

// ReconFlag 2 (LoadDateFromDir, :1453-1485): stacks, status and angles from the saved
// buffer%03d.phimap files.  The y angle is the file's y angle (the reference reloads
// the x angle into both).
ctdm_status load_saved(const ctdm_job_file &jb, int R, ctdm_job_result &r, Stacks &S)
{
    const int F = count_files(jb.save_dir, "buffer");
    if (F < 1) return fail_io(std::string("no buffer*.phimap files in ") + jb.save_dir);
    const long rr = (long)R * R;
    r.frames = F;
    S.ph.assign((size_t)F * rr, 0.f);
    S.am.assign((size_t)F * rr, 0.f);
    S.status.assign(F, 1);
    S.angx.assign(F, 0.f);
    S.angy.assign(F, 0.f);
    std::vector<float> ph, am;
    char name[64];
    for (int k = 1; k <= F; k++) {
        snprintf(name, sizeof name, "buffer%03d.phimap", k);
        const std::string path = join(jb.save_dir, name);
        int status = 0, sx = 0, sy = 0;
        double ax = 0, ay = 0;
        ctdm_status st = ctdm_read_phimap(path.c_str(), &status, &ax, &ay, &sx, &sy, nullptr, nullptr);
        if (st != CTDM_OK) return st;
        if (sx != sy || sx > 8192) return fail_invalid(("job: " + path + " is not a square map").c_str());
        if (jb.resize_flag == 1 && sx < R)
            return fail_invalid(("job: " + path + " is smaller than the R x R window").c_str());
        ph.resize((size_t)sx * sx);
        am.resize((size_t)sx * sx);
        st = ctdm_read_phimap(path.c_str(), &status, &ax, &ay, &sx, &sy, ph.data(), am.data());
        if (st != CTDM_OK) return st;
        if (k == 1) r.n_holo = sx;
        S.status[k - 1] = status;
        if (!status) r.rejected++;
        S.angx[k - 1] = (float)ax;
        S.angy[k - 1] = (float)ay;
        combine_to_stack(ph.data(), am.data(), sx, R, jb.resize_flag, S.ph.data(), S.am.data(), k - 1);
    }
    return CTDM_OK;
}

}  // namespace

extern "C" ctdm_status ctdm_run_job(const ctdm_job_file *job, ctdm_job_result *result)
{
    if (!job) return fail_invalid("ctdm_run_job: job is NULL");
    const ctdm_job_file jb = *job;
    ctdm_status st = check_job(jb);
    if (st != CTDM_OK) return st;
    ctdm_job_result r;
    memset(&r, 0, sizeof r);
    const int R = jb.size_type ? 512 : 256;
    r.recon_size = R;
    Stacks S;
    st = jb.recon_flag == 2 ? load_saved(jb, R, r, S) : process_frames(jb, R, r, S);
    if (result) *result = r;
    if (st != CTDM_OK) return st;
    // 3-D reconstruction of the frames that passed (:1230-1242)
    const int recon_frames = r.frames - r.rejected;
    if (jb.recon_flag >= 1 && recon_frames > 1) {
        const int k = refresh_stack(S.ph, S.am, S.status, S.angx, S.angy, (long)R * R);
        ctdm_set_recon_globals(R, jb.n_med, jb.wavelength_nm, jb.camera_pixel_um, jb.mag, jb.iter_time, jb.recon_save,
                               jb.save_dir);
        st = batch_recon(S.ph.data(), S.am.data(), S.angx.data(), S.angy.data(), k);
        if (st != CTDM_OK) return st;
        r.recon_frames = k;
    }
    if (result) *result = r;
    clear_error();
    return CTDM_OK;
}

// ---------------------------------------------------------------- reference-named entry points
extern "C" void HilbertTransform(char *SPDir, char *BGDir, char *AngDir, char *SaveDir, int rowPts[], int colPts[],
                                 int rowSize, int colSize, int StartNo, int SpaceNo, int EndNo)
{
    (void)rowSize; (void)colSize; (void)StartNo; (void)SpaceNo; (void)EndNo;
    ctdm_job_file j = g_job;
    if ((SPDir && !set_path(j.sp_dir, SPDir)) || (BGDir && !set_path(j.bg_dir, BGDir)) ||
        (AngDir && !set_path(j.ang_dir, AngDir)) || (SaveDir && !set_path(j.save_dir, SaveDir))) {
        fail_invalid("HilbertTransform: a folder path is 256 characters or longer");
        return;
    }
    if (rowPts) { j.row_pts[0] = rowPts[0]; j.row_pts[1] = rowPts[1]; }
    if (colPts) { j.col_pts[0] = colPts[0]; j.col_pts[1] = colPts[1]; }
    ctdm_run_job(&j, nullptr);
}

extern "C" int scriptFileRead(char *script)
{
    if (!script) return 0;
    FILE *fp = fopen(script, "rb");
    if (!fp) return 0;
    std::string first_err;
    char entry[1024];
    while (fscanf(fp, "%1023s", entry) == 1) {
        ctdm_job_file j;
        if (ctdm_parse_job_file(entry, &j) != CTDM_OK) {
            if (first_err.empty()) first_err = ctdm_last_error();
            continue;
        }
        g_job = j;
        HilbertTransform(j.sp_dir, j.bg_dir, j.ang_dir, j.save_dir, j.row_pts, j.col_pts,
                         j.row_pts[1] - j.row_pts[0] + 1, j.col_pts[1] - j.col_pts[0] + 1, 1, 1, 1);
        if (first_err.empty() && ctdm_last_error()[0]) first_err = ctdm_last_error();
    }
    fclose(fp);
    if (first_err.empty()) clear_error();
    else fail_io(first_err);
    return 1;
}

extern "C" float AngCal_GPU(float *src, int sizeX, int sizeY, int frame, int totalFrame)
{
    (void)frame; (void)totalFrame;
    if (sizeX != sizeY) {
        fail_invalid("AngCal_GPU: square images only");
        return NAN;
    }
    float a = NAN;
    if (ctdm_angle_from_image(src, sizeX, g_job.n_med, g_job.wavelength_nm, g_job.mag, g_job.camera_pixel_um, &a,
                              nullptr) != CTDM_OK)
        return NAN;
    return a;
}

extern "C" bool checkArray(float *array2D, float limitSTD, float limitRange, int size)
{
    if (!array2D || size < 1) return true;
    return check_array(array2D, size, limitSTD, limitRange);
}
