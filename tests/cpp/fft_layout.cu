// Prints the exchange layout of the register FFTs
// (alignment_projects_gb300/csrc/aln_fft_reg.cuh) for every radix and team
// padding the library instantiates, one line per transform:
//   N R PADK T SMEM  ns b c  ns b c ...
// (one ns b c triple per exchange, in order: buffer index i + c (i >> b)).
// Host code only: it runs without a GPU.
#include <cstdio>

#include "aln_fft_reg.cuh"

template <int N, int R, int PADK>
static void show()
{
    using F = RegFFT<N, -1, R, PADK>;
    static_assert(F::SMEM == regfft_smem(N, R, PADK), "SMEM");
    std::printf("%d %d %d %d %d", N, R, PADK, F::T, F::SMEM);
    int ns = 1;
    if (F::R2 > 1) {
        std::printf("  1 %d %d", xpad_shift(1, R, F::T, PADK), xpad_mul(1, R, F::T));
        ns = F::R2;
    }
    for (int p = 0; p + 1 < F::P; ++p, ns *= R)
        std::printf("  %d %d %d", ns, xpad_shift(ns, R, F::T, PADK), xpad_mul(ns, R, F::T));
    std::printf("\n");
}

// every power of two N >= R at radix R, padding PADK
template <int R, int PADK, int N = R>
static void all_lengths()
{
    if constexpr (N <= ALN_MAX_N) {
        show<N, R, PADK>();
        all_lengths<R, PADK, N * 2>();
    }
}

int main()
{
    all_lengths<2, 4>();
    all_lengths<4, 4>();
    all_lengths<8, 4>();
    all_lengths<16, 4>();
    // the row pass's small teams (padding per T points)
    all_lengths<16, 3>();
    all_lengths<8, 1>();
    all_lengths<8, 2>();
    all_lengths<8, 3>();
    all_lengths<4, 1>();
    all_lengths<4, 2>();
    all_lengths<4, 3>();
    return 0;
}
