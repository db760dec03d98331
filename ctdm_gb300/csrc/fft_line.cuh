// Batched in-shared-memory Stockham FFT over lines.
//
// A CTA holds B lines of length L in shared memory, element p of line b at
// buf[b * LP + p] (LP = L plus a pad that keeps 64-bit accesses of a half-warp
// on distinct banks).  Each radix stage gathers R strided points per butterfly
// into registers, applies the stage twiddles, runs an in-register radix-R DFT
// and scatters back in Stockham (self-sorting) order, so the output is in
// natural order without a bit-reversal pass.  Threads are mapped b-fastest:
// tid -> (b = tid % B, t = tid / B), T threads per line, and every thread keeps
// a register tile of E = L / T points through all stages.
//
// Register-resident ends: the first stage of a transform reads points
// j + r * (L / R0) and the last stage writes points j + r * (L / Rlast) for the
// butterflies j = t + T q of the thread.  A kernel may therefore load the first
// stage straight from global memory and store the last one straight back
// (skipping shared memory), and when a transform is followed by another one
// whose radix order is reversed, the second starts from the registers the first
// ended in.
//
// Row mapping (TF = true): tid -> (t = tid % T, b = tid / T), lanes spread along
// one line, for lines that are contiguous in global memory (a warp's register-end
// loads and stores are then unit-stride).  Point p of line b sits at
// buf[b * (L + L/16) + p + p/16]: one pad slot per 16 points keeps the stride-R
// scatters of the early stages on distinct banks.
//
// Conventions (cuFFT C2C as used by the reference, cTDM/FFT.cu:697-838):
// forward exp(-2 pi i k n / L), inverse exp(+2 pi i k n / L), both unnormalised.
// Twiddles come from a per-length table tw[e] = exp(-2 pi i e / L) computed in
// double on the host.
#pragma once
#include "ctdm_common.cuh"

namespace fftl {

// ---------------------------------------------------------------- radix DFTs
template <bool INV>
__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3)
{
    float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = cmul_mi<INV>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

// exp(-+ 2 pi i k / 8) for k = 1, 3
template <bool INV>
__device__ __forceinline__ float2 w8(float2 a, int k)
{
    const float h = 0.70710678118654752440f;
    float2 w = (k == 1) ? make_float2(h, INV ? h : -h) : make_float2(-h, INV ? h : -h);
    return cmul(a, w);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2 *a)
{
    // radix-2 decimation in time over two radix-4 DFTs
    float2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
    float2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    o1 = w8<INV>(o1, 1);
    o2 = cmul_mi<INV>(o2);
    o3 = w8<INV>(o3, 3);
    a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
    a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
    a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
    a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
}

// x exp(-+ 2 pi i 2/16) = h (1 -+ i) and x exp(-+ 2 pi i 6/16) = h (-1 -+ i): two adds and
// two multiplies each
template <bool INV>
__device__ __forceinline__ float2 mul_w16_2(float2 a)
{
    const float h = 0.70710678118654752440f;
    return INV ? make_float2(h * (a.x - a.y), h * (a.x + a.y)) : make_float2(h * (a.x + a.y), h * (a.y - a.x));
}
template <bool INV>
__device__ __forceinline__ float2 mul_w16_6(float2 a)
{
    const float h = 0.70710678118654752440f;
    return INV ? make_float2(-h * (a.x + a.y), h * (a.x - a.y)) : make_float2(h * (a.y - a.x), -h * (a.x + a.y));
}

template <bool INV>
__device__ __forceinline__ void dft16(float2 *a)
{
    // 16 = 4 x 4 (n = 4 n1 + n2, k = k1 + 4 k2): four 4-point DFTs over n1, the twiddles
    // W16^(n2 k1) (W^4 = -+i free, W^2 and W^6 by mul_w16_*), four 4-point DFTs over n2;
    // 160 real operations against 172 for two 8-point halves
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    float2 b[16];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
        b[4 * n2 + 0] = a[n2];
        b[4 * n2 + 1] = a[4 + n2];
        b[4 * n2 + 2] = a[8 + n2];
        b[4 * n2 + 3] = a[12 + n2];
        dft4<INV>(b[4 * n2 + 0], b[4 * n2 + 1], b[4 * n2 + 2], b[4 * n2 + 3]);
    }
    const float2 w1 = make_float2(c1, INV ? s1 : -s1);
    const float2 w3 = make_float2(s1, INV ? c1 : -c1);
    const float2 w9 = make_float2(-c1, INV ? -s1 : s1);
    b[5] = cmul(b[5], w1);
    b[6] = mul_w16_2<INV>(b[6]);
    b[7] = cmul(b[7], w3);
    b[9] = mul_w16_2<INV>(b[9]);
    b[10] = cmul_mi<INV>(b[10]);
    b[11] = mul_w16_6<INV>(b[11]);
    b[13] = cmul(b[13], w3);
    b[14] = mul_w16_6<INV>(b[14]);
    b[15] = cmul(b[15], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        float2 x0 = b[k1], x1 = b[4 + k1], x2 = b[8 + k1], x3 = b[12 + k1];
        dft4<INV>(x0, x1, x2, x3);
        a[k1] = x0;
        a[k1 + 4] = x1;
        a[k1 + 8] = x2;
        a[k1 + 12] = x3;
    }
}

template <bool INV>
__device__ __forceinline__ void dft3(float2 *a)
{
    const float s3 = 0.86602540378443864676f;
    float2 t1 = cadd(a[1], a[2]);
    float2 d = csub(a[1], a[2]);
    // forward: (a1 - a2) * (-i s3); inverse: * (+i s3)
    float2 t2 = INV ? make_float2(-s3 * d.y, s3 * d.x) : make_float2(s3 * d.y, -s3 * d.x);
    float2 m = make_float2(a[0].x - 0.5f * t1.x, a[0].y - 0.5f * t1.y);
    a[0] = cadd(a[0], t1);
    a[1] = cadd(m, t2);
    a[2] = csub(m, t2);
}

template <int R, bool INV>
__device__ __forceinline__ void dftR(float2 *a)
{
    if constexpr (R == 2) dft2<INV>(a[0], a[1]);
    else if constexpr (R == 3) dft3<INV>(a);
    else if constexpr (R == 4) dft4<INV>(a[0], a[1], a[2], a[3]);
    else if constexpr (R == 8) dft8<INV>(a);
    else if constexpr (R == 16) dft16<INV>(a);
}

// ---------------------------------------------------------------- one stage
// Shared-memory position of point p: padded line stride LP (column mapping) or
// one pad slot per 16 points (row mapping).
template <int L, int LP, bool TF>
struct Lay {
    static constexpr int LINE = TF ? L + L / 16 : LP;
    __device__ static __forceinline__ int at(int p) { return TF ? p + (p >> 4) : p; }
};

// Register tile v[E], E = L / T, viewed as PER butterflies of R points.
template <int L, int T, int LP, int R, bool TF = false>
__device__ __forceinline__ void gather(const float2 *buf, float2 *v, int b, int t)
{
    using Y = Lay<L, LP, TF>;
    constexpr int NB = L / R, PER = NB / T;
    const float2 *line = buf + b * Y::LINE;
#pragma unroll
    for (int q = 0; q < PER; q++)
#pragma unroll
        for (int r = 0; r < R; r++) v[q * R + r] = line[Y::at(t + T * q + r * NB)];
}

template <int L, int T, bool INV, int NS, int R>
__device__ __forceinline__ void compute(float2 *v, const float2 *__restrict__ tw, int t)
{
    constexpr int NB = L / R, PER = NB / T;
    static_assert(NB % T == 0, "threads per line must divide the butterfly count");
#pragma unroll
    for (int q = 0; q < PER; q++) {
        if constexpr (NS > 1) {
            const int k = (t + T * q) % NS;
#pragma unroll
            for (int r = 1; r < R; r++) {
                const float2 w = __ldg(&tw[r * k * (L / (NS * R))]);
                v[q * R + r] = INV ? cmulc(v[q * R + r], w) : cmul(v[q * R + r], w);
            }
        }
        dftR<R, INV>(v + q * R);
    }
}

template <int L, int T, int LP, int NS, int R, bool TF = false>
__device__ __forceinline__ void scatter(float2 *buf, const float2 *v, int b, int t)
{
    using Y = Lay<L, LP, TF>;
    constexpr int NB = L / R, PER = NB / T;
    float2 *line = buf + b * Y::LINE;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        const int j = t + T * q;
        const int base = (j / NS) * NS * R + (j % NS);
#pragma unroll
        for (int r = 0; r < R; r++) line[Y::at(base + r * NS)] = v[q * R + r];
    }
}

// Barrier between the shared-memory exchanges of a transform.  Under the row mapping a
// line's T threads are consecutive, so with T dividing 32 a line lies inside one warp and
// touches only its own slots: a warp barrier orders its exchanges.  The column mapping
// spreads a line over the CTA and needs the CTA barrier.  (Exchanges with data written
// or read by another mapping, GATHER0 / SCATTER_LAST, keep the CTA barrier.)
template <bool TF, int T, bool LOCAL>
__device__ __forceinline__ void line_sync()
{
    if constexpr (TF && LOCAL && T <= 32 && (32 % T) == 0) __syncwarp();
    else __syncthreads();
}

// Stages in the order given.  GATHER0: the first stage reads shared memory
// (else its inputs are already in v).  SCATTER_LAST: the last stage writes shared
// memory (else its outputs stay in v).
template <int L, int T, int LP, bool INV, bool GATHER0, bool SCATTER_LAST, bool TF, int NS, int R, int... REST>
__device__ __forceinline__ void stages(float2 *buf, float2 *v, const float2 *__restrict__ tw, int b, int t)
{
    constexpr bool first = (NS == 1);
    constexpr bool last = (sizeof...(REST) == 0);
    if constexpr (!first || GATHER0) {
        gather<L, T, LP, R, TF>(buf, v, b, t);
        line_sync<TF, T, !(first && GATHER0)>();
    }
    compute<L, T, INV, NS, R>(v, tw, t);
    if constexpr (!last || SCATTER_LAST) {
        scatter<L, T, LP, NS, R, TF>(buf, v, b, t);
        line_sync<TF, T, !(last && SCATTER_LAST)>();
    }
    if constexpr (!last) stages<L, T, LP, INV, GATHER0, SCATTER_LAST, TF, NS * R, REST...>(buf, v, tw, b, t);
}

// ---------------------------------------------------------------- plans
// A plan: line length L, B lines per CTA, T threads per line and the radix
// sequence.  seq() runs the sequence as listed, seqr() reversed; *_row() are the
// same under the row mapping.  F0 / RV0: first radix of the listed / reversed order
// (the radices at the register-resident ends).
template <int... Rs>
struct Radices {};
template <int A, int... Rest>
struct FirstOf {
    static constexpr int v = A;
};

template <int L_, int B_, int T_, class FWD, class REV>
struct PlanT;
template <int L_, int B_, int T_, int... FW, int... RV>
struct PlanT<L_, B_, T_, Radices<FW...>, Radices<RV...>> {
    static constexpr int L = L_, B = B_, T = T_;
    static constexpr int PAD = (B >= 16) ? 1 : (16 / B);
    static constexpr int LP = L + PAD;
    static constexpr int THREADS = B * T;
    static constexpr int E = L / T;
    static constexpr int F0 = FirstOf<FW...>::v, RV0 = FirstOf<RV...>::v;
    static_assert(E * T == L, "threads per line must divide the length");
    template <bool INV, bool GATHER0, bool SCATTER_LAST>
    __device__ static __forceinline__ void seq(float2 *buf, float2 *v, const float2 *tw)
    {
        stages<L, T, LP, INV, GATHER0, SCATTER_LAST, false, 1, FW...>(buf, v, tw, threadIdx.x % B, threadIdx.x / B);
    }
    template <bool INV, bool GATHER0, bool SCATTER_LAST>
    __device__ static __forceinline__ void seqr(float2 *buf, float2 *v, const float2 *tw)
    {
        stages<L, T, LP, INV, GATHER0, SCATTER_LAST, false, 1, RV...>(buf, v, tw, threadIdx.x % B, threadIdx.x / B);
    }
    template <bool INV>
    __device__ static __forceinline__ void seq_row(float2 *buf, float2 *v, const float2 *tw)
    {
        stages<L, T, LP, INV, false, false, true, 1, FW...>(buf, v, tw, threadIdx.x / T, threadIdx.x % T);
    }
    template <bool INV>
    __device__ static __forceinline__ void seqr_row(float2 *buf, float2 *v, const float2 *tw)
    {
        stages<L, T, LP, INV, false, false, true, 1, RV...>(buf, v, tw, threadIdx.x / T, threadIdx.x % T);
    }
    template <bool INV>
    __device__ static __forceinline__ void run(float2 *buf, const float2 *tw)
    {
        float2 v[E];
        seq<INV, true, true>(buf, v, tw);
    }
};

// Default plan per length (2-D transforms, QPI, DCT, Ewald mapping, and variant 0
// of the volume passes).
template <int L>
struct Plan;
#define FFTL_PLAN(LL, BB, TT, FWD, REV) \
    template <>                         \
    struct Plan<LL> : PlanT<LL, BB, TT, Radices<FWD>, Radices<REV>> {};
#define FFTL_LIST(...) __VA_ARGS__
FFTL_PLAN(16, 64, 4, FFTL_LIST(4, 4), FFTL_LIST(4, 4))
FFTL_PLAN(32, 64, 4, FFTL_LIST(8, 4), FFTL_LIST(4, 8))
FFTL_PLAN(64, 32, 8, FFTL_LIST(8, 8), FFTL_LIST(8, 8))
FFTL_PLAN(128, 32, 8, FFTL_LIST(16, 8), FFTL_LIST(8, 16))
FFTL_PLAN(256, 16, 16, FFTL_LIST(16, 16), FFTL_LIST(16, 16))
FFTL_PLAN(384, 32, 8, FFTL_LIST(16, 8, 3), FFTL_LIST(3, 8, 16))
FFTL_PLAN(512, 16, 16, FFTL_LIST(8, 8, 8), FFTL_LIST(8, 8, 8))
FFTL_PLAN(768, 16, 16, FFTL_LIST(16, 16, 3), FFTL_LIST(3, 16, 16))
FFTL_PLAN(1024, 8, 32, FFTL_LIST(16, 16, 4), FFTL_LIST(4, 16, 16))
FFTL_PLAN(1536, 8, 32, FFTL_LIST(16, 16, 3, 2), FFTL_LIST(2, 3, 16, 16))
FFTL_PLAN(2048, 4, 64, FFTL_LIST(16, 16, 8), FFTL_LIST(8, 16, 16))
#undef FFTL_PLAN
#undef FFTL_LIST

// First radix of the listed (forward) sequence and of the reversed one.
template <int L>
struct Ends {
    static constexpr int F = Plan<L>::F0, Rv = Plan<L>::RV0;
};

// Plan variants of the volume passes, chosen per pass by the autotuner.  Every
// stage's butterfly count L / R must be a multiple of T.
template <int L, int V>
struct PV;
template <int L>
struct PV<L, 0> : Plan<L> {};
template <> struct PV<256, 1> : PlanT<256, 8, 16, Radices<16, 16>, Radices<16, 16>> {};
template <> struct PV<256, 2> : PlanT<256, 16, 32, Radices<8, 4, 8>, Radices<8, 4, 8>> {};
template <> struct PV<384, 1> : PlanT<384, 16, 16, Radices<4, 4, 8, 3>, Radices<3, 8, 4, 4>> {};
template <> struct PV<384, 2> : PlanT<384, 8, 16, Radices<4, 4, 8, 3>, Radices<3, 8, 4, 4>> {};
template <> struct PV<512, 1> : PlanT<512, 16, 32, Radices<8, 8, 8>, Radices<8, 8, 8>> {};
template <> struct PV<512, 2> : PlanT<512, 8, 32, Radices<8, 8, 8>, Radices<8, 8, 8>> {};
template <> struct PV<768, 1> : PlanT<768, 8, 32, Radices<8, 8, 4, 3>, Radices<3, 4, 8, 8>> {};
template <> struct PV<768, 2> : PlanT<768, 16, 32, Radices<8, 8, 4, 3>, Radices<3, 4, 8, 8>> {};

// Point index of register slot i (butterfly q = i / R, point r = i % R) at the
// register-resident end of a sequence whose end radix is R: j + r * (L / R).
template <int L, int T, int R>
__device__ __forceinline__ int slot_pos(int i, int t)
{
    return (t + T * (i / R)) + (i % R) * (L / R);
}

template <int L>
__host__ __device__ constexpr size_t smem_bytes()
{
    return sizeof(float2) * Plan<L>::B * Plan<L>::LP;
}
template <class P>
__host__ __device__ constexpr size_t plan_smem()
{
    return sizeof(float2) * P::B * P::LP;
}
template <class P>
__host__ __device__ constexpr size_t plan_smem_row()
{
    return sizeof(float2) * P::B * (P::L + P::L / 16);
}
// Resident CTAs per SM to ask of the register allocator for a plan: `want` for
// register tiles of up to 16 points, fewer for longer tiles.
template <class P>
__host__ __device__ constexpr int plan_min_ctas(int want)
{
    // two-stage tiles of up to 16 points: `want` x 256 resident threads per SM;
    // longer tiles or three-stage lengths (more twiddles live): 512
    return (P::E <= 16 && P::L <= 256) ? (want * 256 / P::THREADS > 0 ? want * 256 / P::THREADS : 1)
                                       : (P::E <= 32 ? (512 / P::THREADS > 0 ? 512 / P::THREADS : 1) : 1);
}

// Resident CTAs per SM to ask of the register allocator: `want` for register
// tiles of up to 16 points, fewer for the longer tiles so they do not spill.
template <int L>
__host__ __device__ constexpr int min_ctas(int want)
{
    return Plan<L>::E <= 16 ? want : (Plan<L>::E <= 32 ? 2 : 1);
}

// Shared memory of the row mapping.
template <int L>
__host__ __device__ constexpr size_t smem_bytes_row()
{
    return sizeof(float2) * Plan<L>::B * (L + L / 16);
}

}  // namespace fftl

// Dispatch a templated launcher over the supported line lengths.
#define CTDM_DISPATCH_L(Lrt, FN, ...)                  \
    switch (Lrt) {                                     \
    case 16: return FN<16>(__VA_ARGS__);               \
    case 32: return FN<32>(__VA_ARGS__);               \
    case 64: return FN<64>(__VA_ARGS__);               \
    case 128: return FN<128>(__VA_ARGS__);             \
    case 256: return FN<256>(__VA_ARGS__);             \
    case 384: return FN<384>(__VA_ARGS__);             \
    case 512: return FN<512>(__VA_ARGS__);             \
    case 768: return FN<768>(__VA_ARGS__);             \
    case 1024: return FN<1024>(__VA_ARGS__);           \
    case 1536: return FN<1536>(__VA_ARGS__);           \
    case 2048: return FN<2048>(__VA_ARGS__);           \
    default: return cudaErrorInvalidValue;             \
    }
