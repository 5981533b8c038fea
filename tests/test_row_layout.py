"""The row kernel's shared-memory layout, on the CPU.  tests/cpp/row_layout.cu
prints the layout the library is compiled with (aln_row_layout.cuh's
constexpr functions, through nvcc) for every row length the library
instantiates.  This test checks it:

* each team's region holds its staged row bytes (from the region's first
  16-byte boundary), its exchange buffer and its L + 1 bins; regions do not
  overlap and end inside the G * pitch + 16 float2 the launch allocates;
* the lag kernels' team pitch holds the L + 1 bins at padi(k) and the
  inverse transform's exchange buffer, and is odd;
* a bank model of 8-byte shared-memory accesses (a half-warp's 16 threads
  take one wavefront per distinct address on the busiest of the 16 bank
  pairs): the register FFT's exchanges (write and read addresses of
  RegFFT / MixFFT, aln_fft_reg.cuh) and the epilogue's reads of bins kx and
  L - kx for row x % G (k2_rowfft, aln_pipeline.cuh) cost what the layout's
  comment states -- conflict-free but for the split lengths' radix-4
  sub-transforms."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "alignment_projects_gb300", "csrc")


def _nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return n if os.path.exists(n) else None


@pytest.fixture(scope="module")
def layout(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("row_layout") / "row_layout")
    subprocess.check_call([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I" + CSRC, "-o", exe, os.path.join(HERE, "cpp", "row_layout.cu")])
    out = {}
    for ln in subprocess.check_output([exe], text=True).splitlines():
        if ln.startswith("lag "):
            L, pitch, smem = (int(x) for x in ln.split()[1:])
            out.setdefault("lag", {})[L] = dict(pitch=pitch, smem=smem)
            continue
        f = [int(x) for x in ln.split()]
        L, T, G, padk, smem, pitch = f[:6]
        out[L] = dict(T=T, G=G, padk=padk, smem=smem, pitch=pitch, base=f[6:])
        assert len(out[L]["base"]) == G
    return out


def _instantiated_lengths():
    src = open(os.path.join(CSRC, "aln_corr.cu")).read()
    ls = set()
    for name in ("ALN_CASES_L", "ALN_CASES_LMIX"):
        m = re.search(r"#define %s\(X\)(.*)" % name, src)
        ls |= {int(x) for x in re.findall(r"X\((\d+)\)", m.group(1))}
    return ls


def test_every_row_length_is_covered(layout):
    assert _instantiated_lengths() <= set(layout)
    assert _instantiated_lengths() <= set(layout["lag"])


def test_lag_pitch(layout):
    for L, d in layout["lag"].items():
        padi_last = L + (L >> 4)            # padi(L), the last bin's slot
        assert d["pitch"] > padi_last + 1 and d["pitch"] >= d["smem"], L
        assert d["pitch"] % 2 == 1, L


def test_regions_hold_their_data_and_stay_apart(layout):
    for L, d in layout.items():
        if L == "lag":
            continue
        need = max(L + 1, d["smem"], (4 * L + 30 + 8 + 7) // 8)
        assert d["pitch"] >= need + 15, L
        b = d["base"]
        for g in range(d["G"]):
            # staged bytes start at the region's first 16-byte boundary
            # (at most 8 bytes in; regions start on 8 bytes)
            first16 = (b[g] * 8 + 15) // 16 * 16
            assert first16 + 4 * L + 30 <= (b[g] + need) * 8, (L, g)
            if g + 1 < d["G"]:
                assert b[g] + need <= b[g + 1], (L, g)
        assert b[-1] + need <= d["G"] * d["pitch"] + 16, L


def _odd_part(n):
    while n % 2 == 0:
        n //= 2
    return n


def _fft_radix(n):
    return 16 if n >= 512 else (8 if n >= 8 else n)


def _sub(L, T):
    """(N1, N2, R) of the row transform: RegFFT (N1 = 1) or MixFFT."""
    n1 = _odd_part(L)
    return n1, L // n1, (L // n1) // T


def _cost(addrs):
    per = {}
    for a in set(addrs):
        per[a % 16] = per.get(a % 16, 0) + 1
    return max(per.values())


def _exchange_factor(L, d):
    """Wavefronts of one warp's exchange accesses over the conflict-free
    count, for the teams of the CTA's first warp."""
    T, padk, base = d["T"], d["padk"], d["base"]
    n1, n2, R = _sub(L, T)
    P = (n2.bit_length() - 1) // (R.bit_length() - 1)
    R2 = n2 // R ** P
    thr = list(range(32))
    team = [x // T for x in thr]
    t = [x % T for x in thr]
    pad = lambda i: i + (i >> padk)
    tot = ideal = 0

    def access(idx):
        nonlocal tot, ideal
        for h in (0, 16):
            tot += _cost([base[team[x]] + pad(idx[x]) for x in range(h, h + 16)])
            ideal += 1

    ns = 1
    if R2 > 1:
        m = R // R2
        for q in range(m):
            for s in range(R2):
                access([(tt + q * T) * R2 + s for tt in t])
        for r in range(R):
            access([tt + r * T for tt in t])
        ns = R2
    for p in range(P):
        if p + 1 < P:
            for r in range(R):
                access([(tt - (tt & (ns - 1))) * R + (tt & (ns - 1)) + r * ns for tt in t])
            for r in range(R):
                access([tt + r * T for tt in t])
        ns *= R
    return tot / ideal if ideal else 1.0


def _epilogue_factor(L, d):
    """Wavefronts of the epilogue's reads Z[kx] and Z[L - kx] (thread x:
    row x % G, bins x / G + m T) over the conflict-free count, first item."""
    T, G, base = d["T"], d["G"], d["base"]
    tot = ideal = 0
    for h in range(0, G * T, 16):
        xs = range(h, h + 16)
        for hi in (False, True):
            addrs = []
            for x in xs:
                kx = x // G
                k = (L - kx) % L if hi else kx
                addrs.append(base[x % G] + k)
            tot += _cost(addrs)
            ideal += 1
    return tot / ideal


# the split lengths' radix-4 sub-transforms keep strided exchange writes
# that one pad slot per 16 (or per T) does not separate
EXCHANGE_FACTOR = {160: 1.25, 320: 1.75, 384: 4 / 3, 640: 4 / 3, 768: 1.5, 1280: 1.5,
                   1536: 1.25}


def test_bank_model(layout):
    for L, d in layout.items():
        if L == "lag":
            continue
        ex = _exchange_factor(L, d)
        assert ex <= EXCHANGE_FACTOR.get(L, 1.0) + 1e-9, (L, ex)
        ep = _epilogue_factor(L, d)
        assert ep == 1.0, (L, ep)
