// aln_row_layout.cuh -- shared-memory layouts of the row kernels
// (aln_pipeline.cuh): the row pass k2_rowfft (team size, teams per CTA,
// exchange padding, region pitch and region starts) and the lag kernels'
// team pitch.  Host and device code both use these (the launches size their
// shared memory from rowfft_pitch and lag_pitch).
#pragma once

#include "aln_fft_reg.cuh"

// threads per CTA of the row kernels: >= 256, four teams when teams are large
__host__ __device__ constexpr int rowfft_threads(int T) { return T * 4 > 512 ? 512 : (T * 4 < 256 ? 256 : T * 4); }

// Per-thread radix of the row transforms: 16 from 128 points up (fewer
// shared-memory exchange passes: the row kernel is bound by them), the
// register FFT's default below.
__host__ __device__ constexpr int rowfft_radix(int L) { return L >= 128 ? 16 : fft_radix(L); }

// Shared-memory layout of the row kernel.  Each team owns one row's region:
// the row's staged bytes, then the transform's exchange buffer, then the
// row's L bins (plain index), reused in that order.  Region starts are
// shifted (by under 16 float2) onto chosen bank pairs.  Teams of T <= 8
// threads share a half-warp with 16 / T - 1 neighbours: the teams of a
// half-warp sit T bank pairs apart -- their consecutive and odd-strided
// accesses then fall on distinct banks -- and each aligned group of 16
// regions starts on 16 distinct bank pairs (an epilogue half-warp reads one
// bin of 16 rows).  Teams of 32 threads or more leave G < 16 rows per CTA,
// and an epilogue half-warp reads 16 / G consecutive bins of G rows: those
// regions start 16 / G bank pairs apart.  The split lengths take the
// transform in decimation-in-frequency order (a team's threads read
// consecutive pixel pairs), and teams of T = 2, 4 and 8 threads pad the
// exchange buffer by one slot per T points (per 16 for larger teams).
// (Modelled on 8-byte half-warp wavefronts: the odd-pitch layout with
// padding per 16 cost 1.75-4x the conflict-free count on the 160- and
// 192-point rows; padding per 8 cost 1.5x on teams of 2 and 4 threads, and
// regions one bank pair apart 2-4x on the epilogue reads of G < 16 rows.)
template <int L>
__host__ __device__ constexpr int rowfft_T() { return fft_team(L, rowfft_radix(L)); }
template <int L>
__host__ __device__ constexpr int rowfft_padk()
{
    return rowfft_T<L>() >= 16 ? 4 : rowfft_T<L>() >= 8 ? 3 : rowfft_T<L>() >= 4 ? 2
         : rowfft_T<L>() >= 2 ? 1 : 4;
}

// The row transform of half-length L: the power-of-two RegFFT at
// rowfft_radix(L), or for L = 3 * 2^k, 5 * 2^k (CorrPatches grids) the
// MixFFT split.
template <int L>
using RowFFT = FFTOf<L, -1, true, rowfft_radix(L), rowfft_padk<L>()>;

// float2 per team region: the bins, the exchange buffer and the staged
// bytes (<= 4L + 38 with the 16-byte alignment) all fit, plus the shift.
template <int L>
__host__ __device__ constexpr int rowfft_pitch()
{
    constexpr int a = L + 1, b = RowFFT<L>::SMEM, c = (4 * L + 38 + 7) / 8;
    return (a > b ? (a > c ? a : c) : (b > c ? b : c)) + 15;
}
// start of team g's region (float2); a CTA needs G * pitch + 16 float2
template <int L>
__host__ __device__ constexpr int rowfft_base(int g)
{
    constexpr int T = rowfft_T<L>(), P = rowfft_pitch<L>();
    constexpr int G = rowfft_threads(T) / T;
    const int want = T < 16 ? ((g % (16 / T)) * T + g / (16 / T)) % 16
                   : G >= 16 ? g % 16 : (g * (16 / G)) % 16;
    return g * P + ((want - g * P) % 16 + 16) % 16;
}

// CTAs per SM the row kernel is compiled for: 5 up to 256-point
// power-of-two rows (48 registers, no spills), 64 registers per thread for
// longer rows and for the split lengths (12-24 points per thread).
template <int L>
__host__ __device__ constexpr int rowfft_minb()
{
    return odd_part(L) == 1 && L <= 256 ? 5 : 1024 / rowfft_threads(rowfft_T<L>());
}

// float2 per team in the lag kernels (k2_lagrow, k2_lagimg, k2_lagp2i): the
// team's L + 1 bins at padi(k) and the inverse transform's exchange buffer
// (both from the region's start), rounded up to an odd count.  The CTA
// loads the rows with one bin per thread and the teams (rows) fastest, G
// consecutive threads writing bin k of G rows at k + g * pitch: an odd pitch
// puts those on G distinct 8-byte banks (an even one had two threads on
// every bank).
template <int L>
__host__ __device__ constexpr int lag_pitch()
{
    return (padded(L) + 2 > FFTOf<L, +1>::SMEM ? padded(L) + 2 : FFTOf<L, +1>::SMEM) | 1;
}
