// Goldstein branch-cut unwrapping (y-h-Lin/cTDM cudaGoldsteinUnwrap2D,
// cTDM/Goldstein.cu:5-50).
//
// Residues (cudaPhaseResidues :52-103) are computed per pixel with the
// reference's float/double expression, so the charges are bit-exact.
//
// Branch cuts: the reference launches cudaBC (:128-201) with one thread per
// residue and no synchronisation between them, so its cut mask depends on
// scheduling.  The deterministic specification used here executes the same
// body for the residues one after another in raster order (the FP64 oracle
// does the same).  One warp per map scans the residues; for each it searches
// the box perimeters of radius r = 1, 2, ... with 32 cells per step (ballot
// picks the first cell that fires in the reference's loop order) and
// rasterises the cut (cuPlaceBranchCutInternal :224-248) lane-parallel.
//
// Flood fill: the reference's CPU FloodFill (:643-1095) visits the active
// ("adjoin") pixels of each sweep in raster order, and a pixel sees the
// updates of pixels visited before it in the same sweep.  That order is
// reproduced exactly without a serial loop: per sweep, which active pixels get
// unwrapped is the least fixed point of a monotone system over their left/upper
// neighbours, the reference neighbour of each follows from it, and values are
// evaluated in dependency rounds; the adjoin set of the next sweep is derived
// from the visiting order.  One CTA per map, state bits in shared memory.
#include <cmath>

#include "kernels_front.cuh"

namespace ctdm {

// ------------------------------------------------------------ residues
__device__ __forceinline__ float res_term(float a, float b)
{
    const float d = __fsub_rn(a, b);
    const float x = __double2float_rn(__dadd_rn((double)d, CTDM_PI_D));
    const float m = (float)(CTDM_PI_D * 2);
    float r = fmodf(x, m);
    if (r < 0.f) r = __fadd_rn(r, m);
    return __double2float_rn(__dsub_rn((double)r, CTDM_PI_D));
}

// The same wrapped difference in float alone, with `sure` cleared when a - b + pi lies
// within 1e-4 (relative to 2 pi) of a multiple of 2 pi, where the rounding of the exact
// expression decides between -pi and +pi.  Elsewhere the two differ by a few ulp.
__device__ __forceinline__ float res_term_fast(float a, float b, bool &sure)
{
    const float m = (float)(CTDM_PI_D * 2);
    const float x = (a - b) + (float)CTDM_PI_D;
    const float q = x * (float)(1.0 / (CTDM_PI_D * 2));
    const float k = floorf(q), f = q - k;
    if (f < 1e-4f || f > 1.0f - 1e-4f) sure = false;
    return fmaf(-k, m, x) - (float)CTDM_PI_D;
}

// Charges: the float evaluation decides every pixel whose terms are clear of the wrap
// boundaries and whose sum is more than 1e-3 from +-6 (its error is below 1e-5); the
// exact expression of cudaPhaseResidues runs for the rest, so the charges are the same.
__global__ void residues_kernel(const float *__restrict__ phi, int W, int H, int8_t *q)
{
    const int a = blockIdx.z;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const long n = (long)W * H;
    const float *p = phi + a * n;
    int8_t v = 0;
    if (x != W - 1 && y != H - 1) {
        const float p00 = p[x + (long)W * y], p10 = p[(x + 1) + (long)W * y];
        const float p11 = p[(x + 1) + (long)W * (y + 1)], p01 = p[x + (long)W * (y + 1)];
        bool sure = true;
        const float t0 = res_term_fast(p00, p10, sure) + res_term_fast(p10, p11, sure) +
                         res_term_fast(p11, p01, sure) + res_term_fast(p01, p00, sure);
        if (sure && fabsf(fabsf(t0) - 6.0f) > 1e-3f) {
            v = t0 >= 6.0f ? 1 : (t0 <= -6.0f ? -1 : 0);
        } else {
            const float r1 = res_term(p00, p10), r2 = res_term(p10, p11);
            const float r3 = res_term(p11, p01), r4 = res_term(p01, p00);
            const float t = __fadd_rn(__fadd_rn(__fadd_rn(r1, r2), r3), r4);
            v = t >= 6.0f ? 1 : (t <= -6.0f ? -1 : 0);
        }
    }
    q[a * n + x + (long)W * y] = v;
}

cudaError_t goldstein_residues(const float *phi, int A, int W, int H, int8_t *charges, cudaStream_t s)
{
    dim3 block(32, 8), grid((W + 31) / 32, (H + 7) / 8, A);
    residues_kernel<<<grid, block, 0, s>>>(phi, W, H, charges); note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ branch cuts
// cuPlaceBranchCutInternal with its unsigned bounds test, lanes over the fill steps.
__device__ void place_cut(volatile uint8_t *cut, int W, unsigned r1, unsigned c1, unsigned r2, unsigned c2, int lane)
{
    if (lane == 0) {
        cut[r1 + (unsigned)W * c1] = 1;
        cut[r2 + (unsigned)W * c2] = 1;
    }
    const float dR = (float)(int)(r2 - r1);
    const float dC = (float)(int)(c2 - c1);
    const float radius = __fsqrt_rn(__fadd_rn(__fmul_rn(dR, dR), __fmul_rn(dC, dC)));
    const float ct = __fdiv_rn(dR, radius);
    const float st = __fdiv_rn(dC, radius);
    const int nr = __float2int_rn(radius);
    const unsigned rlo = min(r1, r2) - 1u, rhi = max(r1, r2) + 1u;
    const unsigned clo = min(c1, c2) - 1u, chi = max(c1, c2) + 1u;
    for (int ii = 1 + lane; ii <= nr; ii += 32) {
        const unsigned rf = r1 + (unsigned)__float2int_rn(__fmul_rn((float)ii, ct));
        const unsigned cf = c1 + (unsigned)__float2int_rn(__fmul_rn((float)ii, st));
        if (rf > rlo && rf < rhi && cf > clo && cf < chi) cut[rf + (unsigned)W * cf] = 1;
    }
    __syncwarp();
}

// Cell s of the perimeter of the box [m1, m2] x [n1, n2] in cudaBC's loop order:
// column m1 (all rows), interior columns (rows n1 and n2), column m2 (all rows).
__device__ __forceinline__ void seq_cell(unsigned s, unsigned m1, unsigned m2, unsigned n1, unsigned n2, unsigned Hc,
                                         unsigned Wc, unsigned &mm, unsigned &nn)
{
    if (s < Hc) { mm = m1; nn = n1 + s; return; }
    s -= Hc;
    if (s < 2 * (Wc - 2)) { mm = m1 + 1 + s / 2; nn = (s & 1) ? n2 : n1; return; }
    s -= 2 * (Wc - 2);
    mm = m2;
    nn = n1 + s;
}

__global__ void __launch_bounds__(32) cuts_kernel(const int8_t *__restrict__ charges, int W, int H, uint8_t *cuts,
                                                  int8_t *work)
{
    const int a = blockIdx.x, lane = threadIdx.x;
    const long n = (long)W * H;
    volatile int8_t *masked = work + a * n;
    volatile uint8_t *cut = cuts + a * n;
    const int8_t *q = charges + a * n;
    for (long p = lane; p < n; p += 32) {
        masked[p] = q[p];
        cut[p] = 0;
    }
    __syncwarp();
    int maxBox = 901;
    const int half = (int)floorf((float)(W / 2));
    if (half < maxBox) maxBox = half;
    unsigned maxR = (unsigned)maxBox;
    const unsigned hr = (unsigned)__float2int_rn(__fmul_rn((float)W, 0.5f));
    if (hr < maxR) maxR = hr;
    const unsigned uW = (unsigned)W, uH = (unsigned)H;
    for (long base = 0; base < n; base += 32) {
        const long pl = base + lane;
        const int v = pl < n ? masked[pl] : 0;
        unsigned pend = __ballot_sync(0xffffffffu, v != 0);
        while (pend) {
            const int l = __ffs(pend) - 1;
            pend &= pend - 1;
            const unsigned idx = (unsigned)(base + l);
            __syncwarp();
            if (masked[idx] == 0) continue;   // cleared by an earlier residue
            const unsigned i = idx % uW, j = idx / uW;
            if (i <= 0 || i >= uW - 1 || j <= 0 || j >= uH - 1) {
                if (lane == 0) {
                    cut[idx] = 1;
                    masked[idx] = 0;
                }
                __syncwarp();
            }
            for (unsigned r = 1; r < maxR; r++) {
                const unsigned m1 = i - r, n1 = j - r;
                const unsigned m2 = min(i + r, uW - 1), n2 = min(j + r, uH - 1);
                if (m1 > m2 || n1 > n2) break;   // unsigned wrap: this box and all larger ones are empty
                const unsigned Hc = n2 - n1 + 1, Wc = m2 - m1 + 1;
                const unsigned total = 2 * Hc + 2 * (Wc - 2);
                bool found = false;
                for (unsigned s0 = 0; s0 < total && !found; s0 += 32) {
                    const unsigned sidx = s0 + lane;
                    int cond = 0;
                    unsigned mm = 0, nn = 0;
                    if (sidx < total) {
                        seq_cell(sidx, m1, m2, n1, n2, Hc, Wc, mm, nn);
                        if (mm <= 0 || mm >= uW - 1) cond = 1;
                        else if (nn <= 0 || nn >= uH - 1) cond = 2;
                        else if ((int)masked[idx] * (int)masked[mm + uW * nn] == -1) cond = 3;
                    }
                    const unsigned hit = __ballot_sync(0xffffffffu, cond != 0);
                    if (!hit) continue;
                    found = true;
                    const int f = __ffs(hit) - 1;
                    const unsigned fmm = __shfl_sync(0xffffffffu, mm, f);
                    const unsigned fnn = __shfl_sync(0xffffffffu, nn, f);
                    const int fc = __shfl_sync(0xffffffffu, cond, f);
                    if (fc == 1) {
                        place_cut(cut, W, i, j, fmm, j, lane);
                        if (lane == 0) { masked[idx] = 0; masked[i + uW * fnn] = 0; }
                    } else if (fc == 2) {
                        place_cut(cut, W, i, j, i, fnn, lane);
                        if (lane == 0) { masked[idx] = 0; masked[fmm + uW * j] = 0; }
                    } else {
                        place_cut(cut, W, i, j, fmm, fnn, lane);
                        if (lane == 0) { masked[idx] = 0; masked[fmm + uW * fnn] = 0; }
                    }
                    __syncwarp();
                    // the rest of column fmm is still visited with the charge spent:
                    // only the edge branches can fire there
                    const bool full = (fmm == m1 || fmm == m2);
                    const unsigned step = full ? 1u : (n2 - n1);
                    for (unsigned nn2 = fnn + step; step != 0 && nn2 <= n2; nn2 += step) {
                        if (fmm <= 0 || fmm >= uW - 1) {
                            place_cut(cut, W, i, j, fmm, j, lane);
                            if (lane == 0) masked[i + uW * nn2] = 0;
                        } else if (nn2 <= 0 || nn2 >= uH - 1) {
                            place_cut(cut, W, i, j, i, nn2, lane);
                            if (lane == 0) masked[fmm + uW * j] = 0;
                        }
                        __syncwarp();
                    }
                }
                if (found) break;
            }
        }
    }
}

cudaError_t goldstein_cuts(const int8_t *charges, int A, int W, int H, uint8_t *cuts, int8_t *work, cudaStream_t s)
{
    cuts_kernel<<<A, 32, 0, s>>>(charges, W, H, cuts, work); note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ flood fill
// State bits per pixel.  The active ("adjoin") set of each sweep is an unsorted
// list: the visiting order matters only through index comparisons, and two
// consecutive lists are identical exactly when they have the same length and
// every entry of the new one was in the old one (F_PREV).
enum : unsigned {
    F_CUT = 1u, F_UB = 2u, F_PREV = 4u, F_LIST = 8u, F_NEW = 16u, F_CAND = 32u, F_READY = 64u, F_MARK = 128u
};
constexpr int FF_THREADS = 256;

__device__ __forceinline__ unsigned byte_or(uint8_t *p, unsigned bits)
{
    const uintptr_t addr = reinterpret_cast<uintptr_t>(p);
    unsigned *w = reinterpret_cast<unsigned *>(addr & ~(uintptr_t)3);
    const unsigned sh = 8u * (unsigned)(addr & 3);
    return (atomicOr(w, bits << sh) >> sh) & 0xffu;
}

// neighbour k of p in the reference's order: below (p+1), above (p-1), right
// (p+W), left (p-W); the reference's "row" index is the fast one.
__device__ __forceinline__ bool neighbour(int p, int k, int W, int H, int &nb)
{
    const int rr = p % W, cc = p / W;
    switch (k) {
    case 0: nb = p + 1; return rr + 1 <= W - 1;
    case 1: nb = p - 1; return rr - 1 >= 0;
    case 2: nb = p + W; return cc + 1 <= H - 1;
    default: nb = p - W; return cc - 1 >= 0;
    }
}

// Unwrapped state of nb when p is visited: list pixels before p carry their
// state after their own visit (F_NEW), every other pixel its old state.
__device__ __forceinline__ bool ub_at_visit(const uint8_t *st, int nb, int p)
{
    const unsigned s = st[nb];
    if ((s & F_LIST) && nb < p) return (s & F_NEW) != 0;
    return (s & F_UB) != 0;
}

// ref + atan2(sin D, cos D), D = phi - ref: the wrap of D into (-pi, pi] computed
// as D - 2 pi round(D / 2 pi) in double, then rounded to float.  In float: with
// k = rint(D / 2 pi) decided away from the halfway points, D - k fl(2 pi) is a multiple
// of 2^-21 below pi in magnitude, so the first fma is exact and the second rounds
// D - k 2 pi once, the double expression's value; the double form runs only near the
// halfway points (GB300's FP64 divide made it most of the fill's arithmetic).
__device__ __forceinline__ float unwrap_from(float ref, float ph)
{
    const float d = __fsub_rn(ph, ref);
    const float qf = d * (float)(0.5 / CTDM_PI_D);
    const float kf = rintf(qf);
    if (fabsf(fabsf(qf - kf) - 0.5f) > 1e-5f && fabsf(d) < 1e6f) {
        const float p1 = (float)(2 * CTDM_PI_D);
        const float p2 = (float)(2 * CTDM_PI_D - (double)(float)(2 * CTDM_PI_D));
        const float a = fmaf(-kf, p1, d);
        return __fadd_rn(ref, fmaf(-kf, p2, a));
    }
    const double dd = (double)d;
    const double k = rint(__ddiv_rn(dd, 2.0 * CTDM_PI_D));
    const float dp = __double2float_rn(__dsub_rn(dd, __dmul_rn(k, 2.0 * CTDM_PI_D)));
    return __fadd_rn(ref, dp);
}

struct FFLists {
    int *cur, *nxt, *prev, *ref;
    float *nv;
};

// One sweep over the list (use_cuts: main loop; else the final cut-pixel fill,
// which ignores cuts and makes no marks).  Marks append to lists.nxt.
__device__ void sweep(uint8_t *st, const FFLists &ls, int L, int *nnext, const float *ph, float *o, int W, int H,
                      bool use_cuts)
{
    const int t = threadIdx.x;
    const int *list = ls.cur;
    // candidates from states that cannot change before the visit
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        unsigned s = st[p];
        bool cand = false;
        for (int k = 0; k < 4; k++) {
            int nb;
            if (!neighbour(p, k, W, H, nb)) continue;
            const unsigned sn = st[nb];
            if (use_cuts && (sn & F_CUT)) continue;
            if (sn & F_UB) cand = true;
        }
        if (cand) s |= F_CAND | F_NEW;
        if (s & F_UB) s |= F_NEW;
        st[p] = (uint8_t)s;
    }
    __syncthreads();
    // least fixed point over the left / upper neighbours visited earlier
    for (int guard = 0; guard <= L; guard++) {
        bool changed = false;
        for (int e = t; e < L; e += FF_THREADS) {
            const int p = list[e];
            const unsigned s = st[p];
            if (s & F_CAND) continue;
            bool cand = false;
            for (int k = 1; k < 4; k += 2) {
                int nb;
                if (!neighbour(p, k, W, H, nb)) continue;
                const unsigned sn = st[nb];
                if (use_cuts && (sn & F_CUT)) continue;
                if ((sn & F_LIST) && (sn & F_NEW)) cand = true;
            }
            if (cand) {
                st[p] = (uint8_t)(s | F_CAND | F_NEW);
                changed = true;
            }
        }
        if (!__syncthreads_or(changed)) break;
    }
    // reference neighbour (first unwrapped in visiting order) and the values whose
    // reference is not recomputed in this sweep
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        const unsigned s = st[p];
        if (!(s & F_CAND)) continue;
        int chosen = -1;
        for (int k = 0; k < 4 && chosen < 0; k++) {
            int nb;
            if (!neighbour(p, k, W, H, nb)) continue;
            if (use_cuts && (st[nb] & F_CUT)) continue;
            if (ub_at_visit(st, nb, p)) chosen = nb;
        }
        ls.ref[e] = chosen;
    }
    __syncthreads();
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        const unsigned s = st[p];
        if (!(s & F_CAND)) continue;
        const int nb = ls.ref[e];
        const unsigned sn = st[nb];
        const bool dep = (sn & F_LIST) && nb < p && (sn & F_CAND);
        if (!dep) {
            ls.nv[p] = unwrap_from(o[nb], ph[p]);
            st[p] = (uint8_t)(s | F_READY);
        }
    }
    __syncthreads();
    // dependency rounds: a value computed in a round is published (F_READY) only
    // after the round's barrier, so a reader never sees the flag before the value.
    // F_PREV is unused during a sweep and marks "computed in this round".
    for (int guard = 0; guard <= L; guard++) {
        bool pending = false;
        for (int e = t; e < L; e += FF_THREADS) {
            const int p = list[e];
            const unsigned s = st[p];
            if (!(s & F_CAND) || (s & F_READY)) continue;
            const int nb = ls.ref[e];
            if (st[nb] & F_READY) {
                ls.nv[p] = unwrap_from(ls.nv[nb], ph[p]);
                st[p] = (uint8_t)(s | F_PREV);
            } else {
                pending = true;
            }
        }
        __syncthreads();
        for (int e = t; e < L; e += FF_THREADS) {
            const int p = list[e];
            const unsigned s = st[p];
            if (s & F_PREV) st[p] = (uint8_t)((s & ~F_PREV) | F_READY);
        }
        if (!__syncthreads_or(pending)) break;
    }
    // adjoin marks for the next sweep: a visit marks each usable neighbour that is
    // not unwrapped at that time; a list pixel keeps only the marks made after its
    // own visit.  The first mark of a pixel appends it to the next list.
    if (use_cuts) {
        for (int e = t; e < L; e += FF_THREADS) {
            const int p = list[e];
            for (int k = 0; k < 4; k++) {
                int nb;
                if (!neighbour(p, k, W, H, nb)) continue;
                const unsigned sn = st[nb];
                if (sn & F_CUT) continue;
                if (ub_at_visit(st, nb, p)) continue;
                if (!(sn & F_LIST) || nb < p) {
                    if (!(byte_or(st + nb, F_MARK) & F_MARK)) ls.nxt[atomicAdd(nnext, 1)] = nb;
                }
            }
        }
    }
    __syncthreads();
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        const unsigned s = st[p];
        if (s & F_CAND) o[p] = ls.nv[p];
        st[p] = (uint8_t)((s & (F_CUT | F_MARK)) | ((s & F_NEW) ? F_UB : 0u) | F_PREV);
    }
    __syncthreads();
}

template <bool SMEM>
__global__ void __launch_bounds__(FF_THREADS) floodfill_kernel(const uint8_t *__restrict__ cuts,
                                                              const float *__restrict__ phi, int W, int H, float *out,
                                                              uint8_t *gstate, int *lists, int *status)
{
    extern __shared__ uint8_t sstate[];
    __shared__ int s_ok, s_nnext;
    const int a = blockIdx.x, t = threadIdx.x;
    const long n = (long)W * H;
    uint8_t *st = SMEM ? sstate : gstate + a * n;
    const uint8_t *cut = cuts + a * n;
    const float *ph = phi + a * n;
    float *o = out + a * n;
    int *base = lists + a * 5 * n;
    FFLists ls;
    ls.cur = base;
    ls.nxt = base + n;
    ls.prev = base + 2 * n;
    ls.ref = base + 3 * n;
    ls.nv = reinterpret_cast<float *>(base + 4 * n);
    int nbc_local = 0;
    for (long p = t; p < n; p += FF_THREADS) {
        st[p] = cut[p] ? (uint8_t)F_CUT : (uint8_t)0;
        o[p] = 0.f;
        nbc_local += cut[p] != 0;
    }
    const int nbc = __syncthreads_count(nbc_local > 0);
    if (t == 0) {
        // seed (FloodFill :656-691): walk the diagonal from (W/2, 2) off the cuts,
        // then seed at the transposed coordinates as the reference does
        int xr = W / 2, yr = 2;
        int ok = xr < W && yr < H;
        while (ok && cut[xr + (long)W * yr] == 1) {
            xr++;
            yr++;
            if (xr >= W || yr >= H) ok = 0;
        }
        const int rowRef = yr, colRef = xr;
        if (ok && (rowRef >= W || colRef >= H)) ok = 0;
        int cnt = 0;
        if (ok) {
            const long seed = rowRef + (long)W * colRef;
            const long nbs[4] = {seed - 1, seed + 1, seed - W, seed + W};
            const bool okn[4] = {rowRef > 0, rowRef < W - 1, colRef > 0, colRef < H - 1};
            for (int k = 0; k < 4; k++)
                if (okn[k]) {
                    st[nbs[k]] |= F_MARK;
                    ls.nxt[cnt++] = (int)nbs[k];
                }
            st[seed] |= F_UB;
            o[seed] = ph[seed];
        }
        s_ok = ok;
        s_nnext = cnt;
    }
    __syncthreads();
    if (!s_ok) {
        if (t == 0) status[a] = 2;
        return;
    }
    int L1 = 0, Lprev = 0, countLimit = 0, stat = 0;
    bool abort_fill = false;
    for (int outer = 0; outer < 4; outer++) {
        __syncthreads();
        if (s_nnext == 0) break;
        if (countLimit >= 2) { stat = 2; break; }
        int term = 0;
        while (countLimit < 2) {
            if (++term > 5000) { stat = 1; abort_fill = true; break; }
            // the marked pixels become this sweep's list
            int *tmp = ls.prev;
            ls.prev = ls.cur;
            ls.cur = ls.nxt;
            ls.nxt = tmp;
            __syncthreads();
            const int L2 = s_nnext;
            __syncthreads();
            if (t == 0) s_nnext = 0;
            bool all_prev = true;
            for (int e = t; e < L2; e += FF_THREADS) {
                const int p = ls.cur[e];
                const unsigned s = st[p];
                all_prev &= (s & F_PREV) != 0;
                st[p] = (uint8_t)((s & ~F_MARK) | F_LIST);
            }
            const bool same = __syncthreads_and(all_prev);
            if (L1 == L2) {
                if (same) countLimit++;
            } else {
                countLimit = 0;
            }
            for (int e = t; e < Lprev; e += FF_THREADS) {
                const int p = ls.prev[e];
                st[p] = (uint8_t)(st[p] & ~F_PREV);
            }
            __syncthreads();
            sweep(st, ls, L2, &s_nnext, ph, o, W, H, true);
            L1 = L2;
            Lprev = L2;
        }
        if (abort_fill) break;
    }
    if (!abort_fill && nbc > 0) {
        // final fill of the cut pixels that adjoin unwrapped ones, plus any pixel still
        // marked (only when the sweeps stalled)
        __syncthreads();
        for (int e = t; e < Lprev; e += FF_THREADS) {
            const int p = ls.cur[e];
            st[p] = (uint8_t)(st[p] & ~F_PREV);
        }
        __syncthreads();
        if (t == 0) s_nnext = 0;
        __syncthreads();
        for (long p = t; p < n; p += FF_THREADS) {
            const unsigned s = st[p];
            const int rr = (int)(p % W), cc = (int)(p / W);
            bool add = (s & F_MARK) != 0;
            if (!add && (s & F_CUT) && rr >= 1 && rr <= W - 2 && cc >= 1 && cc <= H - 2)
                add = !(st[p + 1] & F_CUT) || !(st[p - 1] & F_CUT) || !(st[p - W] & F_CUT) || !(st[p + W] & F_CUT);
            if (add) ls.nxt[atomicAdd(&s_nnext, 1)] = (int)p;
        }
        __syncthreads();
        const int L2 = s_nnext;
        for (int e = t; e < L2; e += FF_THREADS) {
            const int p = ls.nxt[e];
            st[p] = (uint8_t)((st[p] & ~F_MARK) | F_LIST);
        }
        int *tmp = ls.cur;
        ls.cur = ls.nxt;
        ls.nxt = tmp;
        __syncthreads();
        sweep(st, ls, L2, &s_nnext, ph, o, W, H, false);
    }
    if (t == 0) status[a] = stat;
}

cudaError_t goldstein_floodfill(const uint8_t *cuts, const float *phi, int A, int W, int H, float *out, uint8_t *state,
                                int *lists, int *status, cudaStream_t s)
{
    const long n = (long)W * H;
    if (n <= 96 * 1024) {
        const size_t smem = (size_t)((n + 3) & ~3L);
        cudaError_t e = cudaFuncSetAttribute(floodfill_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        floodfill_kernel<true><<<A, FF_THREADS, smem, s>>>(cuts, phi, W, H, out, state, lists, status); note_launch();
    } else {
        floodfill_kernel<false><<<A, FF_THREADS, 0, s>>>(cuts, phi, W, H, out, state, lists, status); note_launch();
    }
    return cudaGetLastError();
}

}  // namespace ctdm
