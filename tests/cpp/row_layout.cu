// Prints the row kernels' shared-memory layouts
// (alignment_projects_gb300/csrc/aln_row_layout.cuh) for every row length
// the library instantiates, one line per length for the row pass:
//   L T G padk smem pitch base(0) .. base(G-1)
// (T threads per team, G teams per CTA, exchange padding i + (i >> padk),
// exchange buffer float2, region pitch float2, region starts float2), and
// one for the lag kernels:
//   lag L pitch smem
// (team pitch float2, the inverse transform's exchange buffer float2).
// Host code only: it runs without a GPU.
#include <cstdio>

#include "aln_row_layout.cuh"

template <int L>
static void show()
{
    constexpr int T = rowfft_T<L>();
    constexpr int G = rowfft_threads(T) / T;
    std::printf("%d %d %d %d %d %d", L, T, G, rowfft_padk<L>(), RowFFT<L>::SMEM,
                rowfft_pitch<L>());
    for (int g = 0; g < G; ++g)
        std::printf(" %d", rowfft_base<L>(g));
    std::printf("\n");
    std::printf("lag %d %d %d\n", L, lag_pitch<L>(), FFTOf<L, +1>::SMEM);
}

int main()
{
    show<8>(); show<16>(); show<32>(); show<64>(); show<128>(); show<256>();
    show<512>(); show<1024>(); show<2048>(); show<4096>();
    show<80>(); show<96>(); show<160>(); show<192>(); show<320>(); show<384>();
    show<640>(); show<768>(); show<1280>(); show<1536>();
    return 0;
}
