"""The register FFTs' index arithmetic (alignment_projects_gb300/csrc/
aln_fft_reg.cuh), restated thread by thread in numpy and checked against
numpy.fft on the CPU.  The restatement follows the kernels' code:

* the twiddle table (filled in aln_ctx_create, aln_corr.cu): every length's
  slots tw[tw_base(N) + N + m] are distinct and inside TW_TOTAL;
* RegFFT<N, DIR, R>: the optional smaller first pass of radix R2, the
  Stockham passes (twiddle index Ns R + r k, exchange write address
  (t - k) R + k + r Ns, read address t + r T), each exchange a permutation
  of the padded buffer that reads no slot it did not write, and thread t's
  slot q holding point t + q T before and after.  Each exchange's padding
  (buffer index i + c (i >> b)) and the buffer size come from the library's
  own constexpr functions: tests/cpp/fft_layout.cu prints them for every
  radix and padding the library instantiates;
* the bank model of those paddings (8-byte accesses, a half-warp's 16
  threads taking one wavefront per distinct address on the busiest of the
  16 bank pairs): no exchange costs more than with one slot per 2^PADK
  points, and radix-8 exchanges of teams of 16 threads or more are
  conflict-free;
* MixFFT<N1, N2, DIR, DIF>: the N1 sub-transforms, twiddles W_N^(a j) from
  the N1 * 2^k table and the odd DFTs with the kernel's formulas, in both
  layouts (in_idx / out_idx);
* the layouts the kernels chain on: a forward transform in one layout and
  an inverse in the other return N x to the slots x came from.

Twiddles are kept in FP64 here (the device table is the same values rounded
to FP32), so the comparison is to FP64 rounding: this checks indices and
signs, not FP32 accuracy, which the GPU parity tests cover."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "alignment_projects_gb300", "csrc")

ALN_MAX_N = 1 << 13                       # aln_fft.cuh: ALN_MAX_LOG 13
TW_POW2_SIZE = 2 * ALN_MAX_N
TW3_BASE = TW_POW2_SIZE
TW3_SIZE = 3 * ALN_MAX_N // 2
TW5_BASE = TW3_BASE + TW3_SIZE
TW5_SIZE = 5 * ALN_MAX_N // 4
TW_TOTAL = TW5_BASE + TW5_SIZE


def odd_part(n):
    while n % 2 == 0:
        n //= 2
    return n


def ilog2(n):
    return n.bit_length() - 1


def tw_base(n):
    o = odd_part(n)
    return 0 if o == 1 else TW3_BASE if o == 3 else TW5_BASE


def fft_radix(n):
    return 16 if n >= 512 else (8 if n >= 8 else n)


def mix_radix(n1, n2):
    if n2 < 4:
        return n2
    if n1 == 3 and n2 <= 64:
        return min(fft_radix(n2), 8)
    return 4


def _table():
    h = np.zeros(TW_TOTAL, np.complex128)
    owner = np.zeros(TW_TOTAL, np.int64)
    h[0] = 1
    for n1 in (1, 3, 5):
        n = n1
        while n <= ALN_MAX_N:
            idx = tw_base(n) + n + np.arange(n)
            assert idx.max() < TW_TOTAL, n
            assert not owner[idx].any(), f"length {n} shares twiddle slots with {owner[idx].max()}"
            owner[idx] = n
            h[idx] = np.exp(-2j * np.pi * np.arange(n) / n)
            n <<= 1
    return h


TW = _table()


_LAYOUT = {}


def layout():
    """(N, R, PADK) -> T, SMEM and the exchanges' (ns, b, c), printed by
    tests/cpp/fft_layout.cu from aln_fft_reg.cuh's constexpr functions;
    built on first use (never at collection), skipped without nvcc."""
    if not _LAYOUT:
        _LAYOUT.update(_build_layout())
    return _LAYOUT


def _build_layout():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    import tempfile
    d = tempfile.mkdtemp(prefix="fft_layout")
    exe = os.path.join(d, "fft_layout")
    subprocess.check_call([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I" + CSRC, "-o", exe, os.path.join(HERE, "cpp", "fft_layout.cu")])
    out = {}
    for ln in subprocess.check_output([exe], text=True).splitlines():
        f = [int(x) for x in ln.split()]
        n, r, padk, T, smem = f[:5]
        ex = [tuple(f[5 + 3 * i:8 + 3 * i]) for i in range((len(f) - 5) // 3)]
        out[(n, r, padk)] = dict(T=T, smem=smem, ex=ex)
    shutil.rmtree(d, ignore_errors=True)
    return out


def test_twiddle_table_layout():
    """Every length's slots are its own, the three tables end where
    TW_TOTAL says, and each table's last length fills its table exactly."""
    assert tw_base(6144) + 2 * 6144 == TW3_BASE + TW3_SIZE
    assert tw_base(5120) + 2 * 5120 == TW5_BASE + TW5_SIZE
    assert 2 * ALN_MAX_N == TW_POW2_SIZE
    assert np.allclose(TW[tw_base(96) + 96 + 1], np.exp(-2j * np.pi / 96))


def dft(v, r, sign):
    """DFT<R, DIR>::run on the last axis: radix-2 splits, natural order."""
    if r == 1:
        return v
    e = dft(v[..., 0::2], r // 2, sign)
    o = dft(v[..., 1::2], r // 2, sign)
    t = o * np.exp(sign * 2j * np.pi * np.arange(r // 2) / r)
    return np.concatenate([e + t, e - t], axis=-1)


def dft_odd(z, n1, sign):
    """DFTOdd<3/5, DIR>::run on the last axis, with the kernel's formulas."""
    x = [z[..., i] for i in range(n1)]
    if n1 == 3:
        s = sign * np.sin(2 * np.pi / 3)
        a, b = x[1] + x[2], x[1] - x[2]
        m = x[0] - 0.5 * a
        ib = 1j * s * b
        out = [x[0] + a, m + ib, m - ib]
    else:
        c1, c2 = np.cos(2 * np.pi / 5), np.cos(4 * np.pi / 5)
        s1, s2 = sign * np.sin(2 * np.pi / 5), sign * np.sin(4 * np.pi / 5)
        a1, b1 = x[1] + x[4], x[1] - x[4]
        a2, b2 = x[2] + x[3], x[2] - x[3]
        m1 = x[0] + c1 * a1 + c2 * a2
        m2 = x[0] + c2 * a1 + c1 * a2
        j1 = 1j * (s1 * b1 + s2 * b2)
        j2 = 1j * (s2 * b1 - s1 * b2)
        out = [x[0] + a1 + a2, m1 + j1, m2 + j2, m2 - j2, m1 - j1]
    return np.stack(out, axis=-1)


class Exchange:
    """The team's exchange buffer of `size` float2; exchange e indexes slot i
    at i + c_e (i >> b_e).  Checks that one exchange's writes are distinct,
    inside the buffer, and that its reads only see written slots."""

    def __init__(self, n, size, pads):
        self.size = size
        self.n = n
        self.pads = list(pads)
        self.e = 0

    def swap(self, writes, reads):
        """writes: list of (index array, values); reads: list of index arrays."""
        b, c = self.pads[self.e]
        self.e += 1
        pad = lambda i: i + c * (i >> b)
        sm = np.full(self.size, np.nan + 0j)
        seen = np.zeros(self.size, np.int64)
        for idx, val in writes:
            p = pad(idx)
            assert p.max() < self.size
            np.add.at(seen, p, 1)
            sm[p] = val
        assert seen.max() == 1, "two threads write one exchange slot"
        assert seen.sum() == self.n
        out = []
        for idx in reads:
            p = pad(idx)
            assert seen[p].all(), "a thread reads a slot nobody wrote"
            out.append(sm[p])
        return np.stack(out, axis=1)


def regfft(v, n, sign, r, padk=4):
    """RegFFT<N, DIR, R, PADK>::run_impl over all T threads at once;
    v[t, q] is thread t's register slot q.  Exchange paddings and the buffer
    size are the library's (layout())."""
    T = n // r
    P = ilog2(n) // ilog2(r)
    r2 = n // r ** P
    t = np.arange(T)
    lay = layout()[(n, r, padk)]
    ex = Exchange(n, lay["smem"], [(b, c) for _, b, c in lay["ex"]])
    v = v.copy()
    ns = 1
    if r2 > 1:
        m = r // r2
        for q in range(m):
            cols = [q + s * m for s in range(r2)]
            v[:, cols] = dft(v[:, cols], r2, sign)
        writes = []
        for q in range(m):
            j = t + q * T
            for s in range(r2):
                writes.append((j * r2 + s, v[:, q + s * m]))
        assert lay["ex"][ex.e][0] == 1
        v = ex.swap(writes, [t + rr * T for rr in range(r)])
        ns = r2
    for p in range(P):
        k = t & (ns - 1)
        if ns > 1:
            nr = ns * r
            for rr in range(1, r):
                assert (rr * k).max() < nr
                w = TW[nr + rr * k]
                v[:, rr] *= np.conj(w) if sign > 0 else w
        v = dft(v, r, sign)
        if p + 1 < P:
            base = (t - k) * r + k
            assert lay["ex"][ex.e][0] == ns
            v = ex.swap([(base + rr * ns, v[:, rr]) for rr in range(r)],
                        [t + rr * T for rr in range(r)])
        ns *= r
    assert ex.e == len(ex.pads)
    return v


def mix_idx(n1, n2, r, dif, inp):
    """MixFFT::in_idx / out_idx as an index array [t, q]."""
    T = n2 // r
    t = np.arange(T)[:, None]
    q = np.arange(n1 * r)[None, :]
    a = q // r
    j = t + (q - a * r) * T
    natural = j + n2 * a          # x[j + N2 a]
    split = a + n1 * j            # x[a + N1 j]
    return (natural if dif else split) if inp else (split if dif else natural)


def mixfft(v, n1, n2, sign, dif, r, padk=4):
    """MixFFT<N1, N2, DIR, DIF, R, PADK>::run_impl over all threads."""
    T = n2 // r
    n = n1 * n2
    v = v.copy()

    def subs(v):
        for a in range(n1):
            v[:, a * r:(a + 1) * r] = regfft(v[:, a * r:(a + 1) * r], n2, sign, r, padk)

    if not dif:
        subs(v)
    t = np.arange(T)
    for rr in range(r):
        j = t + rr * T
        cols = [a * r + rr for a in range(n1)]
        z = v[:, cols]
        tw = np.stack([TW[tw_base(n) + n + a * j] for a in range(n1)], axis=1)
        assert (n1 - 1) * j.max() < n
        if sign > 0:
            tw = np.conj(tw)
        if not dif:
            z = dft_odd(z * tw, n1, sign)
        else:
            z = dft_odd(z, n1, sign) * tw
        v[:, cols] = z
    if dif:
        subs(v)
    return v


def _ref(x, sign):
    return np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * len(x)


def _check(got, want, n):
    err = np.abs(got - want).max() / max(1.0, np.abs(want).max())
    assert err < 1e-12 * max(1, ilog2(n)), err


POW2 = [1 << k for k in range(1, ilog2(ALN_MAX_N) + 1)]


def row_padk(T):
    """rowfft_padk (aln_row_layout.cuh): one pad slot per T points for teams
    of 2, 4 and 8 threads, per 16 otherwise."""
    return 4 if T >= 16 else 3 if T >= 8 else 2 if T >= 4 else 1 if T >= 2 else 4


@pytest.mark.parametrize("n", POW2)
@pytest.mark.parametrize("sign", [-1, +1])
def test_regfft_layout(n, sign):
    """Every radix (2-16) and team padding the library instantiates for this
    length: slot q of thread t holds x[t + q T] in, X[t + q T] out."""
    rng = np.random.default_rng(n * 7 + sign)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    want = _ref(x, sign)
    done = 0
    for r in (2, 4, 8, 16):
        if r > n:
            continue
        T = n // r
        idx = np.arange(T)[:, None] + np.arange(r)[None, :] * T
        for padk in (1, 2, 3, 4):
            if (n, r, padk) not in layout():
                continue
            got = regfft(x[idx], n, sign, r, padk)
            _check(got, want[idx], n)
            done += 1
    assert done


def _warp_exchanges(n, r):
    """Per exchange of RegFFT<n, ., r>: (ns, write index lists, read index
    lists), one index per thread of the team's first warp."""
    T = n // r
    P = ilog2(n) // ilog2(r)
    r2 = n // r ** P
    t = np.arange(min(T, 32))
    out = []
    ns = 1
    if r2 > 1:
        m = r // r2
        w = [(t + q * T) * r2 + s for q in range(m) for s in range(r2)]
        out.append((1, w, [t + rr * T for rr in range(r)]))
        ns = r2
    for p in range(P):
        if p + 1 < P:
            k = t & (ns - 1)
            w = [(t - k) * r + k + rr * ns for rr in range(r)]
            out.append((ns, w, [t + rr * T for rr in range(r)]))
        ns *= r
    return out


def _wavefronts(idx_lists, b, c):
    """8-byte accesses: per half-warp instruction, the distinct addresses on
    the busiest of the 16 bank pairs; summed, over the conflict-free count."""
    tot = ideal = 0
    for idx in idx_lists:
        a = idx + c * (idx >> b)
        for h in range(0, len(a), 16):
            banks = {}
            for x in set(int(v) for v in a[h:h + 16]):
                banks[x % 16] = banks.get(x % 16, 0) + 1
            tot += max(banks.values())
            ideal += 1
    return tot / ideal


def test_exchange_bank_model():
    """For teams of 16 threads or more (a half-warp inside one team): no
    exchange's padding costs more wavefronts than one slot per 2^PADK
    points, and every radix-8 exchange is conflict-free (one slot per 16
    left the second exchange at 1.5x)."""
    checked = 0
    for (n, r, padk), lay in layout().items():
        if lay["T"] < 16 or padk != 4:   # teams of 16+ threads always pad with 4
            continue
        exs = _warp_exchanges(n, r)
        assert [e[0] for e in exs] == [e[0] for e in lay["ex"]], (n, r)
        for (ns, w, rd), (_, b, c) in zip(exs, lay["ex"]):
            new = _wavefronts(w + rd, b, c)
            old = _wavefronts(w + rd, padk, 1)
            assert new <= old + 1e-12, (n, r, padk, ns, new, old)
            if r == 8:
                assert new == 1.0, (n, r, padk, ns, new)
            checked += 1
    assert checked


def _mix_lengths():
    out = []
    for n1 in (3, 5):
        n2 = 2
        while n1 * n2 <= ALN_MAX_N:
            out.append((n1, n2))
            n2 *= 2
    return out


@pytest.mark.parametrize("n1,n2", _mix_lengths())
def test_mixfft_layouts(n1, n2):
    """N = 3 * 2^k and 5 * 2^k at the radix mix_radix picks: the DIT layout
    (in x[a + N1 j], out X[j + N2 a]) and the DIF layout (swapped), forward
    and inverse."""
    n = n1 * n2
    r = mix_radix(n1, n2)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for sign in (-1, +1):
        want = _ref(x, sign)
        for dif in (False, True):
            iin = mix_idx(n1, n2, r, dif, True)
            iout = mix_idx(n1, n2, r, dif, False)
            got = mixfft(x[iin], n1, n2, sign, dif, r, row_padk(n2 // r))
            _check(got, want[iout], n)


@pytest.mark.parametrize("n", [80, 96, 160, 192, 320, 384, 640, 768, 1280, 1536, 128, 256, 512])
def test_row_transform_chains_with_lag_transform(n):
    """The row pass's forward transform (decimation in frequency for split
    lengths) and the lag pass's inverse (decimation in time) meet in one
    layout: a pointwise product between them needs no exchange, and the
    round trip returns N x to the slots x came from."""
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    n1 = odd_part(n)
    if n1 == 1:
        rf = 16 if n >= 128 else fft_radix(n)      # rowfft_radix
        ri = fft_radix(n)                          # FFTOf<L, +1>
        T = n // rf
        idx = np.arange(T)[:, None] + np.arange(rf)[None, :] * T
        spec = regfft(x[idx], n, -1, rf, row_padk(T))
        # the lag pass gets its input through memory by bin index
        flat = np.empty(n, np.complex128)
        flat[idx] = spec
        Ti = n // ri
        idx_i = np.arange(Ti)[:, None] + np.arange(ri)[None, :] * Ti
        back = regfft(flat[idx_i], n, +1, ri)
        _check(back, n * x[idx_i], n)
        return
    n2 = n // n1
    r = mix_radix(n1, n2)
    padk = row_padk(n2 // r)
    assert (mix_idx(n1, n2, r, True, False) == mix_idx(n1, n2, r, False, True)).all()
    iin = mix_idx(n1, n2, r, True, True)
    spec = mixfft(x[iin], n1, n2, -1, True, r, padk)
    back = mixfft(spec, n1, n2, +1, False, r, 4)
    assert (mix_idx(n1, n2, r, False, False) == iin).all()
    _check(back, n * x[iin], n)
