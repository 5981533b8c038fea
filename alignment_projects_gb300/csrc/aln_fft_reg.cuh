// aln_fft_reg.cuh -- register-resident FP32 FFTs for sm_103a.
//
// A "team" of T = N/R threads computes one complex FFT of length N (a power
// of two).  Thread t holds R points in registers, v[r] = x[t + r*T].  Each
// Stockham pass is an R-point DFT in registers (radix 2/4/8/16 built from
// radix-2 splits with exact constants), preceded by twiddles from the device
// table tw[N' + m] = exp(-2 pi i m / N'); between passes the team exchanges
// data once through a padded shared-memory buffer, each exchange with its own
// padding (xpad_shift / xpad_mul below) so that neither its strided writes
// nor its consecutive reads share a bank pair within a half-warp.  (An XOR
// swizzle does the same for one layout, and ran slower in the 512-point
// column kernel: its per-access address arithmetic took registers and
// spilled.)  When N
// is not a power of R the first pass has a smaller radix R2 = N / R^P and
// each thread runs R/R2 of its butterflies.  After the last pass thread t
// holds X[t + r*T]: the same layout as the input, so a forward transform, a
// pointwise product and an inverse transform chain without any exchange.
//
// Conventions: forward sign -1, inverse +1, both unnormalised (FFTW's).
#pragma once

#include "aln_fft.cuh"

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }
__host__ __device__ constexpr int ipowc(int b, int e) { return e == 0 ? 1 : b * ipowc(b, e - 1); }

__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded(int n) { return n + (n >> 4); }


// exp(DIR * 2 pi i k / 16) for k = 0..7 (DIR = -1 forward)
template <int K16, int DIR>
__device__ __forceinline__ float2 mul_w16(float2 x)
{
    constexpr float C1 = 0.92387953251128674f;   // cos(pi/8)
    constexpr float S1 = 0.38268343236508978f;   // sin(pi/8)
    constexpr float H = 0.70710678118654752f;    // sqrt(2)/2
    if constexpr (K16 == 0) {
        return x;
    } else if constexpr (K16 == 4) {
        // forward: * (-i); inverse: * (+i)
        return DIR < 0 ? make_float2(x.y, -x.x) : make_float2(-x.y, x.x);
    } else {
        constexpr float c = K16 == 1 ? C1 : K16 == 2 ? H : K16 == 3 ? S1
                          : K16 == 5 ? -S1 : K16 == 6 ? -H : -C1;
        constexpr float s = K16 == 1 ? S1 : K16 == 2 ? H : K16 == 3 ? C1
                          : K16 == 5 ? C1 : K16 == 6 ? H : S1;
        // w = c + i * DIR * s
        constexpr float ws = DIR < 0 ? -s : s;
        return make_float2(x.x * c - x.y * ws, x.x * ws + x.y * c);
    }
}

// In-place R-point DFT of v[0..R), natural order in and out.
template <int R, int DIR>
struct DFT {
    template <int K>
    __device__ __forceinline__ static void combine(float2 *v, const float2 *e, const float2 *o)
    {
        if constexpr (K < R / 2) {
            const float2 t = mul_w16<K * (16 / R), DIR>(o[K]);
            v[K] = cadd(e[K], t);
            v[K + R / 2] = csub(e[K], t);
            combine<K + 1>(v, e, o);
        }
    }
    __device__ __forceinline__ static void run(float2 *v)
    {
        float2 e[R / 2], o[R / 2];
#pragma unroll
        for (int n = 0; n < R / 2; ++n) {
            e[n] = v[2 * n];
            o[n] = v[2 * n + 1];
        }
        DFT<R / 2, DIR>::run(e);
        DFT<R / 2, DIR>::run(o);
        combine<0>(v, e, o);
    }
};
template <int DIR>
struct DFT<1, DIR> {
    __device__ __forceinline__ static void run(float2 *) {}
};

// Radix used for a given length: 16 for N >= 512, 8 below (keeps T <= 256
// threads and >= 4 threads per team down to N = 32).
__host__ __device__ constexpr int fft_radix(int N) { return N >= 512 ? 16 : (N >= 8 ? 8 : N); }

// Barrier of one team of T threads (team g of the CTA, teams of T
// consecutive threads): a named barrier per team when the team spans whole
// warps (ids 1.. ; 0 is __syncthreads'), the warp's own barrier when teams
// are smaller than a warp (all teams of a warp run the same code path).
// Teams that share no shared-memory data then run apart: one team's wait
// for its loads does not hold the others at the next exchange.
template <int T>
__device__ __forceinline__ void team_sync(int team)
{
    static_assert(T < 32 || T % 32 == 0, "teams are whole warps or within one warp");
    if constexpr (T >= 32)
        asm volatile("bar.sync %0, %1;" ::"r"(team + 1), "r"(T) : "memory");
    else
        __syncwarp();
}

// Exchange padding.  The exchange after a pass whose butterflies are ns
// points apart (ns = 1 after the first pass) has each half-warp write
// groups of ns consecutive slots, ns R apart, and read 16 consecutive slots.
// Slot i sits at buffer index i + c (i >> b):
//   radix 8, teams of T >= 16 threads (a half-warp inside one team) and
//     1 < ns < 16: b = max(4, log2(ns R)), c = ns: each write group lands ns
//     bank pairs after the previous one, so the 16 / ns groups of a
//     half-warp cover the 16 pairs once (one slot per 16 left these
//     exchanges at 1.5x the conflict-free count of 8-byte wavefronts);
//   otherwise b = PADK, c = 1: one slot per 2^PADK points (4 by default,
//     which at radix 16 already moves each write group ns R / 16 = ns bank
//     pairs on; log2 T for the row pass's teams of T = 2, 4, 8 threads,
//     which share a half-warp with neighbour teams placed T bank pairs
//     away).  The split lengths' radix-4 sub-transforms keep one slot per 16
//     (1.25-2.5x): the rule above made their row kernels, capped at 64
//     registers, spill up to 2.6x more.
// b >= 4 keeps each aligned run of 16 slots on 16 distinct bank pairs (the
// reads).  The index grows with i, so every exchange is a permutation.
__host__ __device__ constexpr int xpad_shift(int ns, int R, int T, int PADK)
{
    // log2(ns R) for R = 8 and ns = 2, 4, 8 (a select, not a recursion: ns is
    // a constant only once the pass loop is unrolled)
    return R == 8 && T >= 16 && ns > 1 && ns < 16 ? (ns == 2 ? 4 : ns == 4 ? 5 : 6) : PADK;
}
__host__ __device__ constexpr int xpad_mul(int ns, int R, int T)
{
    return R == 8 && T >= 16 && ns > 1 && ns < 16 ? ns : 1;
}
__host__ __device__ constexpr int xpad_index(int ns, int R, int T, int PADK, int i)
{
    return i + xpad_mul(ns, R, T) * (i >> xpad_shift(ns, R, T, PADK));
}
// float2 per team: the largest index of any exchange of an N-point
// transform at radix R (first pass of radix R2 = N / R^P, then P passes),
// and never less than N + (N >> PADK)
__host__ __device__ constexpr int regfft_smem(int N, int R, int PADK)
{
    const int T = N / R, P = ilog2c(N) / ilog2c(R), R2 = N / ipowc(R, P);
    int m = N + (N >> PADK), ns = 1;
    if (R2 > 1) {
        const int e = xpad_index(1, R, T, PADK, N - 1) + 1;
        m = e > m ? e : m;
        ns = R2;
    }
    for (int p = 0; p + 1 < P; ++p, ns *= R) {
        const int e = xpad_index(ns, R, T, PADK, N - 1) + 1;
        m = e > m ? e : m;
    }
    return m;
}

template <int N, int DIR, int RAD = fft_radix(N), int PADK = 4>
struct RegFFT {
    static constexpr int R = RAD;
    static constexpr int T = N / R;                    // threads per transform
    static constexpr int P = ilog2c(N) / ilog2c(R);    // full radix-R passes
    static constexpr int R2 = N / ipowc(R, P);         // first-pass radix (1: none)
    static constexpr int SMEM = regfft_smem(N, R, PADK);   // float2 per team
    // buffer index of slot i in the exchange after butterflies ns apart
    __device__ __forceinline__ static int xpad(int ns, int i)
    {
        return xpad_index(ns, R, T, PADK, i);
    }
    static constexpr int V = R;                        // points per thread
    // register slot q of thread t holds point t + q T, in and out
    __device__ __forceinline__ static int in_idx(int t, int q) { return t + q * T; }
    __device__ __forceinline__ static int out_idx(int t, int q) { return t + q * T; }

    // All threads of the CTA must call this together (it uses __syncthreads);
    // run_team(..., team) synchronises team `team` alone (team_sync), for
    // kernels whose teams share no shared-memory data around the call.
    __device__ static void run(float2 (&v)[R], float2 *sm, int t,
                               const float2 *__restrict__ tw)
    {
        run_impl<false>(v, sm, t, tw, 0);
    }
    __device__ static void run_team(float2 (&v)[R], float2 *sm, int t,
                                    const float2 *__restrict__ tw, int team)
    {
        run_impl<true>(v, sm, t, tw, team);
    }
    template <bool TEAM>
    __device__ static __forceinline__ void sync(int team)
    {
        if constexpr (TEAM)
            team_sync<T>(team);
        else
            __syncthreads();
    }
    template <bool TEAM>
    __device__ static void run_impl(float2 (&v)[R], float2 *sm, int t,
                                    const float2 *__restrict__ tw, int team)
    {
        int Ns = 1;
        if constexpr (R2 > 1) {
            constexpr int m = R / R2;
#pragma unroll
            for (int q = 0; q < m; ++q) {
                float2 u[R2];
#pragma unroll
                for (int s = 0; s < R2; ++s)
                    u[s] = v[q + s * m];
                DFT<R2, DIR>::run(u);
#pragma unroll
                for (int s = 0; s < R2; ++s)
                    v[q + s * m] = u[s];
            }
            sync<TEAM>(team);
#pragma unroll
            for (int q = 0; q < m; ++q) {
                const int j = t + q * T;
#pragma unroll
                for (int s = 0; s < R2; ++s)
                    sm[xpad(1, j * R2 + s)] = v[q + s * m];
            }
            sync<TEAM>(team);
#pragma unroll
            for (int r = 0; r < R; ++r)
                v[r] = sm[xpad(1, t + r * T)];
            Ns = R2;
        }
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const int k = t & (Ns - 1);
            if (Ns > 1) {
                const int NR = Ns * R;
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    float2 w = __ldg(&tw[NR + r * k]);
                    if (DIR > 0)
                        w.y = -w.y;
                    v[r] = cmul(v[r], w);
                }
            }
            DFT<R, DIR>::run(v);
            if (p + 1 < P) {
                const int base = (t - k) * R + k;
                sync<TEAM>(team);
#pragma unroll
                for (int r = 0; r < R; ++r)
                    sm[xpad(Ns, base + r * Ns)] = v[r];
                sync<TEAM>(team);
#pragma unroll
                for (int r = 0; r < R; ++r)
                    v[r] = sm[xpad(Ns, t + r * T)];
            }
            Ns *= R;
        }
    }
};

// ---------------------------------------------------------------------------
// Lengths N = N1 * 2^k (N1 = 3 or 5)
// ---------------------------------------------------------------------------

// odd factor of n (n > 0)
__host__ __device__ constexpr int odd_part(int n) { return (n & 1) ? n : odd_part(n / 2); }

// Twiddles of the lengths N1 * 2^k sit after the power-of-two table, in
// the same scheme: tw[base(N1) + N + m] = exp(-2 pi i m / N) for every
// N = N1 * 2^k <= ALN_MAX_N.  Each table spans 2 * (its largest N).
constexpr int TW_POW2_SIZE = 2 * ALN_MAX_N;
constexpr int TW3_BASE = TW_POW2_SIZE;
constexpr int TW3_SIZE = 3 * ALN_MAX_N / 2;   // largest N = 3 * ALN_MAX_N / 4
constexpr int TW5_BASE = TW3_BASE + TW3_SIZE;
constexpr int TW5_SIZE = 5 * ALN_MAX_N / 4;   // largest N = 5 * ALN_MAX_N / 8
constexpr int TW_TOTAL = TW5_BASE + TW5_SIZE;

__host__ __device__ constexpr int tw_base(int N)
{
    return odd_part(N) == 1 ? 0 : odd_part(N) == 3 ? TW3_BASE : TW5_BASE;
}

// exp(DIR * 2 pi i m / N), 0 <= m < N, N a power of two or N1 * 2^k
template <int N, int DIR>
__device__ __forceinline__ float2 twn(const float2 *__restrict__ tw, int m)
{
    static_assert(odd_part(N) == 1 || odd_part(N) == 3 || odd_part(N) == 5, "length");
    float2 w = __ldg(&tw[tw_base(N) + N + m]);
    if (DIR > 0)
        w.y = -w.y;
    return w;
}

// In-place N1-point DFT, natural order (N1 = 3, 5), sign DIR.  The constants
// are cos and sin of 2 pi / 3, 2 pi / 5 and 4 pi / 5.
template <int N1, int DIR>
struct DFTOdd;

template <int DIR>
struct DFTOdd<3, DIR> {
    __device__ __forceinline__ static void run(float2 *x)
    {
        constexpr float S = DIR * 0.86602540378443865f;   // DIR * sin(2 pi / 3)
        const float2 a = cadd(x[1], x[2]), b = csub(x[1], x[2]);
        const float2 m = make_float2(x[0].x - 0.5f * a.x, x[0].y - 0.5f * a.y);
        const float2 ib = make_float2(-S * b.y, S * b.x);   // i * DIR * sin * b
        x[0] = cadd(x[0], a);
        x[1] = cadd(m, ib);
        x[2] = csub(m, ib);
    }
};

template <int DIR>
struct DFTOdd<5, DIR> {
    __device__ __forceinline__ static void run(float2 *x)
    {
        constexpr float C1 = 0.30901699437494742f;          // cos(2 pi / 5)
        constexpr float C2 = -0.80901699437494742f;         // cos(4 pi / 5)
        constexpr float S1 = DIR * 0.95105651629515357f;    // DIR * sin(2 pi / 5)
        constexpr float S2 = DIR * 0.58778525229247313f;    // DIR * sin(4 pi / 5)
        const float2 a1 = cadd(x[1], x[4]), b1 = csub(x[1], x[4]);
        const float2 a2 = cadd(x[2], x[3]), b2 = csub(x[2], x[3]);
        const float2 m1 = make_float2(x[0].x + C1 * a1.x + C2 * a2.x,
                                      x[0].y + C1 * a1.y + C2 * a2.y);
        const float2 m2 = make_float2(x[0].x + C2 * a1.x + C1 * a2.x,
                                      x[0].y + C2 * a1.y + C1 * a2.y);
        // i * (S1 b1 + S2 b2) and i * (S2 b1 - S1 b2)
        const float2 j1 = make_float2(-(S1 * b1.y + S2 * b2.y), S1 * b1.x + S2 * b2.x);
        const float2 j2 = make_float2(-(S2 * b1.y - S1 * b2.y), S2 * b1.x - S1 * b2.x);
        x[0] = make_float2(x[0].x + a1.x + a2.x, x[0].y + a1.y + a2.y);
        x[1] = cadd(m1, j1);
        x[4] = csub(m1, j1);
        x[2] = cadd(m2, j2);
        x[3] = csub(m2, j2);
    }
};

// Radix of the power-of-two sub-transforms.  N1 = 3: 8 up to 64 points,
// else 4 (12 points per thread: at radix 8, 24 points per thread, the row
// kernel spilled 180-850 bytes from 128-point sub-transforms up); N1 = 5: 4
// (20 points per thread).
__host__ __device__ constexpr int mix_radix(int N1, int N2)
{
    return N2 < 4 ? N2 : N1 == 3 && N2 <= 64 ? (fft_radix(N2) < 8 ? fft_radix(N2) : 8) : 4;
}

// FFT of length N = N1 * N2 (N2 a power of two) by one Cooley-Tukey split:
// N1 sub-transforms of N2 points (RegFFT, one after another through the
// same exchange buffer), twiddles W_N^(n1 k2) and an N1-point DFT per k2 in
// registers -- no exchange beyond the sub-transforms' own.  A team of
// T = N2 / R threads holds V = N1 R points per thread, slot q = n1 R + r:
//   DIF false (decimation in time):  in  x[n1 + N1 (t + r T)],
//                                    out X[(t + r T) + N2 n1];
//   DIF true (decimation in frequency): the two layouts swapped.
// A forward DIT transform, a pointwise product and an inverse DIF transform
// therefore chain with no exchange, as the power-of-two RegFFT's do.
template <int N1, int N2, int DIR, bool DIF, int RAD = mix_radix(N1, N2), int PADK = 4>
struct MixFFT {
    using Sub = RegFFT<N2, DIR, RAD, PADK>;
    static constexpr int R = Sub::R;
    static constexpr int T = Sub::T;
    static constexpr int V = N1 * R;
    static constexpr int N = N1 * N2;
    static constexpr int SMEM = Sub::SMEM;

    __device__ __forceinline__ static int in_idx(int t, int q)
    {
        const int a = q / R, j = t + (q - a * R) * T;
        return DIF ? j + N2 * a : a + N1 * j;
    }
    __device__ __forceinline__ static int out_idx(int t, int q)
    {
        const int a = q / R, j = t + (q - a * R) * T;
        return DIF ? a + N1 * j : j + N2 * a;
    }
    __device__ static void run(float2 (&v)[V], float2 *sm, int t, const float2 *__restrict__ tw)
    {
        run_impl<false>(v, sm, t, tw, 0);
    }
    __device__ static void run_team(float2 (&v)[V], float2 *sm, int t,
                                    const float2 *__restrict__ tw, int team)
    {
        run_impl<true>(v, sm, t, tw, team);
    }
    template <bool TEAM>
    __device__ static __forceinline__ void subs(float2 (&v)[V], float2 *sm, int t,
                                                const float2 *__restrict__ tw, int team)
    {
#pragma unroll
        for (int a = 0; a < N1; ++a) {
            float2 u[R];
#pragma unroll
            for (int r = 0; r < R; ++r)
                u[r] = v[a * R + r];
            Sub::template run_impl<TEAM>(u, sm, t, tw, team);
#pragma unroll
            for (int r = 0; r < R; ++r)
                v[a * R + r] = u[r];
        }
    }
    template <bool TEAM>
    __device__ static void run_impl(float2 (&v)[V], float2 *sm, int t,
                                    const float2 *__restrict__ tw, int team)
    {
        if constexpr (!DIF)
            subs<TEAM>(v, sm, t, tw, team);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int j = t + r * T;
            float2 z[N1];
#pragma unroll
            for (int a = 0; a < N1; ++a)
                z[a] = v[a * R + r];
            if constexpr (!DIF) {
#pragma unroll
                for (int a = 1; a < N1; ++a)
                    z[a] = cmul(z[a], twn<N, DIR>(tw, a * j));
                DFTOdd<N1, DIR>::run(z);
            } else {
                DFTOdd<N1, DIR>::run(z);
#pragma unroll
                for (int a = 1; a < N1; ++a)
                    z[a] = cmul(z[a], twn<N, DIR>(tw, a * j));
            }
#pragma unroll
            for (int a = 0; a < N1; ++a)
                v[a * R + r] = z[a];
        }
        if constexpr (DIF)
            subs<TEAM>(v, sm, t, tw, team);
    }
};

// The register FFT of length N (a power of two, or N1 * 2^k with N1 = 3, 5):
// RegFFT at radix PRAD, or MixFFT in the DIT (DIF = false) or DIF layout;
// PADK: the exchange padding (RegFFT).
template <bool POW2, int N, int DIR, bool DIF, int PRAD, int PADK>
struct FFTSel {
    using type = RegFFT<N, DIR, PRAD, PADK>;
};
template <int N, int DIR, bool DIF, int PRAD, int PADK>
struct FFTSel<false, N, DIR, DIF, PRAD, PADK> {
    using type = MixFFT<odd_part(N), N / odd_part(N), DIR, DIF,
                        mix_radix(odd_part(N), N / odd_part(N)), PADK>;
};
template <int N, int DIR, bool DIF = false, int PRAD = fft_radix(N), int PADK = 4>
using FFTOf = typename FFTSel<odd_part(N) == 1, N, DIR, DIF, PRAD, PADK>::type;

// Team size of FFTOf<N, ., ., PRAD> without instantiating it.
__host__ __device__ constexpr int fft_team(int N, int PRAD)
{
    return odd_part(N) == 1 ? N / PRAD
                            : (N / odd_part(N)) / mix_radix(odd_part(N), N / odd_part(N));
}
