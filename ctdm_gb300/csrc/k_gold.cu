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

#include "api_internal.h"
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

// Residues of a map in index order, gathered before any cut is placed: lanes load
// CUTS_BATCH bytes each per step, all independent (the charges are mostly zero, and
// one dependent load per 32 pixels made the scan most of the kernel's time).  Pairing
// only clears charges, so a gathered residue that is already paired is skipped.
constexpr int CUTS_BATCH = 32, CUTS_LIST = 2048;

__global__ void __launch_bounds__(32) cuts_kernel(const int8_t *__restrict__ charges, int W, int H, uint8_t *cuts,
                                                  int8_t *work)
{
    __shared__ unsigned s_res[CUTS_LIST];
    const int a = blockIdx.x, lane = threadIdx.x;
    const long n = (long)W * H;
    volatile int8_t *masked = work + a * n;
    volatile uint8_t *cut = cuts + a * n;
    const int8_t *__restrict__ q = charges + a * n;
    int nres = 0;
    for (long base = 0; base < n; base += 32 * CUTS_BATCH) {
        int v[CUTS_BATCH];
#pragma unroll
        for (int k = 0; k < CUTS_BATCH; k++) {
            const long pl = base + 32 * k + lane;
            v[k] = pl < n ? __ldg(q + pl) : 0;
        }
#pragma unroll
        for (int k = 0; k < CUTS_BATCH; k++) {
            const long pl = base + 32 * k + lane;
            if (pl < n) {
                masked[pl] = (int8_t)v[k];
                cut[pl] = 0;
            }
            unsigned pend = __ballot_sync(0xffffffffu, v[k] != 0);
            while (pend) {
                const int l = __ffs(pend) - 1;
                pend &= pend - 1;
                if (lane == 0 && nres < CUTS_LIST) s_res[nres] = (unsigned)(base + 32 * k + l);
                nres++;
            }
        }
    }
    __syncwarp();
    int maxBox = 901;
    const int half = (int)floorf((float)(W / 2));
    if (half < maxBox) maxBox = half;
    unsigned maxR = (unsigned)maxBox;
    const unsigned hr = (unsigned)__float2int_rn(__fmul_rn((float)W, 0.5f));
    if (hr < maxR) maxR = hr;
    const unsigned uW = (unsigned)W, uH = (unsigned)H;
    // more residues than the list holds: walk the map in the same order instead
    const bool listed = nres <= CUTS_LIST;
    const long nsteps = listed ? (long)nres : (n + 31) / 32;
    for (long it = 0; it < nsteps; it++) {
        long base;
        unsigned pend;
        if (listed) {
            base = (long)s_res[it];
            pend = 1u;
        } else {
            base = it * 32;
            const long pl = base + lane;
            pend = __ballot_sync(0xffffffffu, (pl < n ? masked[pl] : 0) != 0);
        }
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

// Lists of one fill: cur / nxt / prev hold pixel indices, ref and nv are indexed by
// the position in cur.  cap is their capacity; a longer list is an overflow.
struct FFLists {
    int *cur, *nxt, *prev, *ref;
    float *nv;
    int cap;
};

// One sweep over the list (use_cuts: main loop; else the final cut-pixel fill,
// which ignores cuts and makes no marks).  Marks append to lists.nxt (past cap they
// are counted, not stored).  Values reach o in two steps: those whose reference was
// unwrapped before the sweep are computed from the old o, then published together
// after a barrier (so every such read sees the old value); the rest are computed in
// dependency rounds from values already published in o.
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
            ls.nv[e] = unwrap_from(o[nb], ph[p]);
            st[p] = (uint8_t)(s | F_READY);
        }
    }
    __syncthreads();
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        if ((st[p] & (F_CAND | F_READY)) == (F_CAND | F_READY)) o[p] = ls.nv[e];
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
                o[p] = unwrap_from(o[nb], ph[p]);
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
                    if (!(byte_or(st + nb, F_MARK) & F_MARK)) {
                        const int q = atomicAdd(nnext, 1);
                        if (q < ls.cap) ls.nxt[q] = nb;
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int e = t; e < L; e += FF_THREADS) {
        const int p = list[e];
        const unsigned s = st[p];
        st[p] = (uint8_t)((s & (F_CUT | F_MARK)) | ((s & F_NEW) ? F_UB : 0u) | F_PREV);
    }
    __syncthreads();
}

// The sweep for lists of at most FF_THREADS pixels, one per thread, with the pixel's
// index, state and neighbours in registers.  It also does the list's conversion
// (MARK -> LIST) and clears F_PREV of the previous list, and returns whether every
// pixel of the list was in the previous one.  Its phases, each ended by a barrier:
//   1. conversion, candidates (from UB and CUT, which no phase of the sweep changes),
//      loads of ph[p] and of the neighbours' old values in o;
//   2. F_PREV cleared on the previous list's pixels outside this list (the owners
//      clear their own), and the fixed point over left / upper neighbours;
//   3. reference neighbour; a value whose reference is not a pixel of this sweep
//      computed from the loaded old value and stored in o at once (every read of an
//      old value was issued before barrier 1);
//   4. dependency rounds, only when some pixel waits on another of this sweep;
//   5. adjoin marks (atomics only); 6. the final states.
// Plain stores to st touch only the owner's pixel except in phase 2, where the
// stores go to pixels outside the list, so no byte store races an atomic or another
// store to the same byte.
__device__ bool sweep_owned(uint8_t *st, const FFLists &ls, int L, int Lprev, int *nnext, const float *ph, float *o,
                            int W, int H)
{
    const int t = threadIdx.x;
    const bool own = t < L;
    int p = 0;
    unsigned s = 0;
    int nbk[4] = {0, 0, 0, 0};
    bool okk[4] = {false, false, false, false};
    float onb[4] = {0.f, 0.f, 0.f, 0.f};
    float phv = 0.f;
    bool all_prev = true;
    if (own) {
        p = ls.cur[t];
#pragma unroll
        for (int k = 0; k < 4; k++) okk[k] = neighbour(p, k, W, H, nbk[k]);
        phv = ph[p];
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (okk[k]) onb[k] = o[nbk[k]];
        s = st[p];
        all_prev = (s & F_PREV) != 0;
        s = (s & ~(F_MARK | F_PREV)) | F_LIST;
        bool cand = false;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!okk[k]) continue;
            const unsigned sn = st[nbk[k]];
            if (sn & F_CUT) continue;
            if (sn & F_UB) cand = true;
        }
        if (cand) s |= F_CAND | F_NEW;
        if (s & F_UB) s |= F_NEW;
        st[p] = (uint8_t)s;
    }
    const bool same = __syncthreads_and(all_prev);
    for (int e = t; e < Lprev; e += FF_THREADS) {
        const int q = ls.prev[e];
        const unsigned r = st[q];
        if (!(r & F_LIST)) st[q] = (uint8_t)(r & ~F_PREV);
    }
    for (int guard = 0; guard <= L; guard++) {
        bool changed = false;
        if (own && !(s & F_CAND)) {
            bool cand = false;
#pragma unroll
            for (int k = 1; k < 4; k += 2) {
                if (!okk[k]) continue;
                const unsigned sn = st[nbk[k]];
                if (sn & F_CUT) continue;
                if ((sn & F_LIST) && (sn & F_NEW)) cand = true;
            }
            if (cand) {
                s |= F_CAND | F_NEW;
                st[p] = (uint8_t)s;
                changed = true;
            }
        }
        if (!__syncthreads_or(changed)) break;
    }
    int kref = -1;
    bool wait_dep = false;
    if (own && (s & F_CAND)) {
        unsigned sref = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (kref >= 0 || !okk[k]) continue;
            const unsigned sn = st[nbk[k]];
            if (sn & F_CUT) continue;
            const bool ub = ((sn & F_LIST) && nbk[k] < p) ? (sn & F_NEW) != 0 : (sn & F_UB) != 0;
            if (ub) {
                kref = k;
                sref = sn;
            }
        }
        // a candidate always has a reference: an unwrapped neighbour made it one
        if (kref >= 0) {
            wait_dep = (sref & F_LIST) && nbk[kref] < p && (sref & F_CAND);
            if (!wait_dep) {
                o[p] = unwrap_from(onb[kref], phv);
                s |= F_READY;
                st[p] = (uint8_t)s;
            }
        }
    }
    if (__syncthreads_or(wait_dep)) {
        for (int guard = 0; guard <= L; guard++) {
            bool done_now = false;
            if (wait_dep) {
                const int nb = nbk[kref];
                if (st[nb] & F_READY) {
                    o[p] = unwrap_from(o[nb], phv);
                    done_now = true;
                }
            }
            __syncthreads();
            if (done_now) {
                s |= F_READY;
                st[p] = (uint8_t)s;
                wait_dep = false;
            }
            if (!__syncthreads_or(wait_dep)) break;
        }
    }
    if (own) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!okk[k]) continue;
            const int nb = nbk[k];
            const unsigned sn = st[nb];
            if (sn & F_CUT) continue;
            const bool ub = ((sn & F_LIST) && nb < p) ? (sn & F_NEW) != 0 : (sn & F_UB) != 0;
            if (ub) continue;
            if (!(sn & F_LIST) || nb < p) {
                if (!(byte_or(st + nb, F_MARK) & F_MARK)) {
                    const int q = atomicAdd(nnext, 1);
                    if (q < ls.cap) ls.nxt[q] = nb;
                }
            }
        }
    }
    __syncthreads();
    if (own) {
        const unsigned r = st[p];
        st[p] = (uint8_t)((r & (F_CUT | F_MARK)) | ((r & F_NEW) ? F_UB : 0u) | F_PREV);
    }
    __syncthreads();
    return same;
}

// Shared-memory lists per fill (each of cur, nxt, prev, ref, nv): a sweep's list is
// the front of the fill, 170 pixels on average and a few hundred at most on 256 x 256
// maps; a fill whose list outgrows the capacity starts over on the global lists.  The
// fill runs beside the reconstruction's loop passes, which lose resident CTAs to a
// larger footprint: 3072 entries (124 KB with the states) slowed the loop by 0.5 ms.
constexpr int FF_SMEM_MAX = 3072, FF_SMEM_CAP = 1024;
static int g_fill_cap = FF_SMEM_CAP;   // set by ctdm_set_fill_list_capacity

// The fill of one map (FloodFill, cTDM/Goldstein.cu:643-1095).  Returns the status (0
// done, 1 sweep limit, 2 no seed) or -1 when a list outgrew ls.cap.
// s_cnt[2]: list lengths; the list of sweep j is counted in s_cnt[j & 1] while sweep j
// counts the next one in s_cnt[(j + 1) & 1].
__device__ int fill_map(uint8_t *st, const uint8_t *cut, const float *ph, float *o, int W, int H, FFLists ls,
                        int *s_ok, int *s_cnt)
{
    const int t = threadIdx.x;
    const long n = (long)W * H;
    int nbc_local = 0;
    for (long p = t; p < n; p += FF_THREADS) {
        st[p] = cut[p] ? (uint8_t)F_CUT : (uint8_t)0;
        o[p] = 0.f;
        nbc_local += cut[p] != 0;
    }
    const int nbc = __syncthreads_count(nbc_local > 0);
    if (t == 0) {
        // seed (FloodFill :656-691): (rowRef, colRef) = (2, W/2), fixed before the
        // reference's diagonal walk off the cuts (:659-663), which therefore changes
        // nothing; the seed may lie on a cut
        const int rowRef = 2, colRef = W / 2;
        const int ok = rowRef < W && colRef < H;
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
        *s_ok = ok;
        s_cnt[0] = cnt;
        s_cnt[1] = 0;
    }
    __syncthreads();
    if (!*s_ok) return 2;
    int L1 = 0, Lprev = 0, countLimit = 0, stat = 0, j = 0;
    bool abort_fill = false;
    for (int outer = 0; outer < 4; outer++) {
        __syncthreads();
        if (s_cnt[j & 1] == 0) break;
        if (countLimit >= 2) { stat = 2; break; }
        int term = 0;
        while (countLimit < 2) {
            if (++term > 5000) { stat = 1; abort_fill = true; break; }
            // the marked pixels become this sweep's list (every sweep ends with a barrier,
            // after which its count is final and the other counter unread)
            int *tmp = ls.prev;
            ls.prev = ls.cur;
            ls.cur = ls.nxt;
            ls.nxt = tmp;
            const int L2 = s_cnt[j & 1];
            if (L2 > ls.cap) return -1;
            int *nnext = &s_cnt[(j + 1) & 1];
            if (t == 0) *nnext = 0;
            bool same;
            if (L2 <= FF_THREADS) {
                same = sweep_owned(st, ls, L2, Lprev, nnext, ph, o, W, H);
            } else {
                bool all_prev = true;
                for (int e = t; e < L2; e += FF_THREADS) {
                    const int p = ls.cur[e];
                    const unsigned s = st[p];
                    all_prev &= (s & F_PREV) != 0;
                    st[p] = (uint8_t)((s & ~F_MARK) | F_LIST);
                }
                same = __syncthreads_and(all_prev);
                for (int e = t; e < Lprev; e += FF_THREADS) {
                    const int p = ls.prev[e];
                    st[p] = (uint8_t)(st[p] & ~F_PREV);
                }
                __syncthreads();
                sweep(st, ls, L2, nnext, ph, o, W, H, true);
            }
            if (L1 == L2) {
                if (same) countLimit++;
            } else {
                countLimit = 0;
            }
            L1 = L2;
            Lprev = L2;
            j++;
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
        int *s_nnext = &s_cnt[0];
        __syncthreads();
        if (t == 0) *s_nnext = 0;
        __syncthreads();
        for (long p = t; p < n; p += FF_THREADS) {
            const unsigned s = st[p];
            const int rr = (int)(p % W), cc = (int)(p / W);
            bool add = (s & F_MARK) != 0;
            if (!add && (s & F_CUT) && rr >= 1 && rr <= W - 2 && cc >= 1 && cc <= H - 2)
                add = !(st[p + 1] & F_CUT) || !(st[p - 1] & F_CUT) || !(st[p - W] & F_CUT) || !(st[p + W] & F_CUT);
            if (add) {
                const int q = atomicAdd(s_nnext, 1);
                if (q < ls.cap) ls.nxt[q] = (int)p;
            }
        }
        __syncthreads();
        const int L2 = *s_nnext;
        if (L2 > ls.cap) return -1;
        for (int e = t; e < L2; e += FF_THREADS) {
            const int p = ls.nxt[e];
            st[p] = (uint8_t)((st[p] & ~F_MARK) | F_LIST);
        }
        int *tmp = ls.cur;
        ls.cur = ls.nxt;
        ls.nxt = tmp;
        __syncthreads();
        sweep(st, ls, L2, s_nnext, ph, o, W, H, false);
    }
    return stat;
}

// One CTA per map.  SMEM: the pixel states (n bytes) and the lists live in shared
// memory, the lists with capacity min(n, FF_SMEM_CAP) and the global ones (5 n ints per
// map) as the fallback; otherwise states and lists are global.
template <bool SMEM>
__global__ void __launch_bounds__(FF_THREADS) floodfill_kernel(const uint8_t *__restrict__ cuts,
                                                              const float *__restrict__ phi, int W, int H, float *out,
                                                              uint8_t *gstate, int *lists, int *status,
                                                              int smem_cap)
{
    extern __shared__ __align__(16) uint8_t sstate[];
    __shared__ int s_ok, s_cnt[2];
    const int a = blockIdx.x;
    const long n = (long)W * H;
    uint8_t *st = SMEM ? sstate : gstate + a * n;
    const uint8_t *cut = cuts + a * n;
    const float *ph = phi + a * n;
    float *o = out + a * n;
    int *base = lists + a * 5 * n;
    FFLists gl;
    gl.cur = base;
    gl.nxt = base + n;
    gl.prev = base + 2 * n;
    gl.ref = base + 3 * n;
    gl.nv = reinterpret_cast<float *>(base + 4 * n);
    gl.cap = (int)n;
    int stat = -1;
    if constexpr (SMEM) {
        const int cap = n < smem_cap ? (int)n : smem_cap;
        int *sl = reinterpret_cast<int *>(sstate + ((n + 15) & ~15L));
        FFLists sm;
        sm.cur = sl;
        sm.nxt = sl + cap;
        sm.prev = sl + 2 * cap;
        sm.ref = sl + 3 * cap;
        sm.nv = reinterpret_cast<float *>(sl + 4 * cap);
        sm.cap = cap;
        stat = fill_map(st, cut, ph, o, W, H, sm, &s_ok, s_cnt);
        __syncthreads();
    }
    if (stat < 0) stat = fill_map(st, cut, ph, o, W, H, gl, &s_ok, s_cnt);
    if (threadIdx.x == 0) status[a] = stat;
}

cudaError_t goldstein_floodfill(const uint8_t *cuts, const float *phi, int A, int W, int H, float *out, uint8_t *state,
                                int *lists, int *status, cudaStream_t s)
{
    const long n = (long)W * H;
    if (n <= 96 * 1024) {
        const int cap = n < g_fill_cap ? (int)n : g_fill_cap;
        const size_t smem = (size_t)(((n + 15) & ~15L) + 5 * sizeof(int) * (size_t)cap);
        cudaError_t e = cudaFuncSetAttribute(floodfill_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        floodfill_kernel<true><<<A, FF_THREADS, smem, s>>>(cuts, phi, W, H, out, state, lists, status, cap);
        note_launch();
    } else {
        floodfill_kernel<false><<<A, FF_THREADS, 0, s>>>(cuts, phi, W, H, out, state, lists, status, 0);
        note_launch();
    }
    return cudaGetLastError();
}

}  // namespace ctdm

extern "C" ctdm_status ctdm_set_fill_list_capacity(int capacity)
{
    if (capacity != 0 && (capacity < 16 || capacity > ctdm::FF_SMEM_MAX))
        return ctdm::fail_invalid("ctdm_set_fill_list_capacity: capacity outside 16..3072");
    ctdm::g_fill_cap = capacity == 0 ? ctdm::FF_SMEM_CAP : capacity;
    return CTDM_OK;
}
