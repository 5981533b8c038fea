// aln_fft_reg.cuh -- register-resident FP32 FFTs for sm_103a.
//
// A "team" of T = N/R threads computes one complex FFT of length N (a power
// of two).  Thread t holds R points in registers, v[r] = x[t + r*T].  Each
// Stockham pass is an R-point DFT in registers (radix 2/4/8/16 built from
// radix-2 splits with exact constants), preceded by twiddles from the device
// table tw[N' + m] = exp(-2 pi i m / N'); between passes the team exchanges
// data once through a padded shared-memory buffer (index i -> i + i/16,
// which keeps the strided Stockham writes free of bank conflicts).  When N
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

// float2 per team in the row kernels: the padded row plus two bins, rounded
// up to an odd count.  The row kernels move data between the teams' rows
// with one bin per thread and the teams (rows) fastest, G consecutive
// threads reading (or writing) bin k of G rows at k + g * pitch: an odd
// pitch puts those on G distinct 8-byte banks (an even one had two threads
// on every bank).  Regions then start on 8 bytes only: the row pass stages
// its input bytes from the region's first 16-byte boundary.
__host__ __device__ constexpr int row_pitch(int L) { return (padded(L) + 2) | 1; }

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

template <int N, int DIR, int RAD = fft_radix(N)>
struct RegFFT {
    static constexpr int R = RAD;
    static constexpr int T = N / R;                    // threads per transform
    static constexpr int P = ilog2c(N) / ilog2c(R);    // full radix-R passes
    static constexpr int R2 = N / ipowc(R, P);         // first-pass radix (1: none)
    static constexpr int SMEM = padded(N);             // float2 per team

    // v: this thread's R points (x[t + r*T]); sm: the team's exchange buffer.
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
                const int j = t + q * T;
#pragma unroll
                for (int s = 0; s < R2; ++s)
                    v[q + s * m] = u[s];
                (void)j;
            }
            sync<TEAM>(team);
#pragma unroll
            for (int q = 0; q < m; ++q) {
                const int j = t + q * T;
#pragma unroll
                for (int s = 0; s < R2; ++s)
                    sm[padi(j * R2 + s)] = v[q + s * m];
            }
            sync<TEAM>(team);
#pragma unroll
            for (int r = 0; r < R; ++r)
                v[r] = sm[padi(t + r * T)];
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
                    sm[padi(base + r * Ns)] = v[r];
                sync<TEAM>(team);
#pragma unroll
                for (int r = 0; r < R; ++r)
                    v[r] = sm[padi(t + r * T)];
            }
            Ns *= R;
        }
    }
};
