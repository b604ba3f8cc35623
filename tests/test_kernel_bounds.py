"""Index arithmetic of the tensor-core convolutions, checked on the CPU for every launch the
denoiser makes (forward and backward-data of each of the 14 layers).

The constants and the layer table are read from the CUDA sources, and the shared-memory
layouts, descriptor address ranges, TMEM columns, TMA box sizes and transaction counts of
salty_gb300/csrc/conv_tc.cu are recomputed here: every operand an MMA reads must lie in
the staged tile, every copy must land inside its stage, the TMEM accumulators of a CTA
must fit its allocation and a CTA's shared memory the 227 KB an SM gives one block."""
import os
import re

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "salty_gb300", "csrc")
SMEM_MAX = 227 * 1024
SMEM_SM = 228 * 1024


def _src(name):
    return open(os.path.join(CSRC, name)).read()


def _const(src, name):
    m = re.search(r"constexpr\s+int\s+" + name + r"\s*=\s*([0-9 *+]+);", src)
    assert m, name
    return eval(m.group(1), {})  # digits, spaces, + and * only (matched above)


@pytest.fixture(scope="module")
def k():
    s = _src("conv_tc.cu")
    c = {n: _const(s, n) for n in ("kTcThreads", "kStrip", "kTmemCols", "kBarBytes", "kMaxStages", "kTmaMmaWarps",
                                   "kTmaHeader", "kTmaMinSmem", "kResidentMaxBytes")}
    c["kHaloW"] = c["kStrip"] + 2
    return c


@pytest.fixture(scope="module")
def launches():
    """(cin, cout, wrows) of every convolution launch: forward, then backward-data (input
    channels = the layer's output channels padded to 16, outputs = its input channels)."""
    u = _src("unet.cu")
    body = re.search(r"const int kLayers\[\]\[3\] = \{(.*?)\};", u, re.S).group(1)
    layers = [tuple(int(x) for x in t) for t in re.findall(r"\{(\d+),\s*(\d+),\s*(\d+)\}", body)]
    assert len(layers) == 14

    def pick_nt(c):
        if c <= 64:
            return c // 8
        for nt in range(6, 1, -1):
            if c % (nt * 8) == 0:
                return nt
        return 2

    def up(a, b):
        return (a + b - 1) // b * b

    out = []
    for cin, cout, _ in layers:
        out.append(("fwd", cin, cout, up(cout, pick_nt(cout) * 8)))
        cpad = up(cout, 16)
        out.append(("bwd", cpad, cin, up(cin, pick_nt(cin) * 8)))
    return out


def rows(k, cout):
    npad = (cout + 15) // 16 * 16
    return min(8, k["kTmemCols"] // npad), npad


def test_cp_async_kernel_layout(k, launches):
    """k_conv3x3_tc: no-swizzle K-major tiles, two stages, 256 TMEM columns."""
    for kind, cin, cout, wrows in launches:
        assert cin % 16 == 0 and cout % 8 == 0 and 16 <= (cout + 15) // 16 * 16 <= 256, (kind, cin, cout)
        R, npad = rows(k, cout)
        hrow = (R + 2) * k["kHaloW"]
        halo = 2 * hrow * 16
        wts = 9 * 2 * npad * 16
        stage = (halo + wts + 127) // 128 * 128
        smem = k["kBarBytes"] + 2 * stage
        assert smem <= SMEM_MAX, (cin, cout, smem)
        # A: row r, tap (ky, kx): 128 core-matrix rows from ((r + ky) * 130 + kx) * 16, plus
        # the second channel octet one plane (LBO) further
        a_end = ((R - 1 + 2) * k["kHaloW"] + 2) * 16 + k["kStrip"] * 16 + hrow * 16
        assert a_end <= halo
        # B: tap t, rows 0..npad-1 from t * 2 * npad * 16, second octet npad * 16 further
        b_end = 8 * 2 * npad * 16 + npad * 16 + npad * 16
        assert b_end <= wts
        assert R * npad <= k["kTmemCols"]
        # descriptor fields: 14 bits of (bytes >> 4)
        assert (hrow * 16) >> 4 < 1 << 14 and (npad * 16) >> 4 < 1 << 14 and (smem >> 4) < 1 << 14
        # at most two CTAs of 256 TMEM columns share an SM's 512
        assert (SMEM_SM // (smem + 1024)) * k["kTmemCols"] <= 512


def test_tma_kernel_layout(k, launches):
    """k_conv3x3_tma: 32-byte-swizzled tiles, 1024-byte aligned stages, one CTA per SM with
    all 512 TMEM columns (two accumulators of R x npad <= 256)."""
    for kind, cin, cout, wrows in launches:
        R, npad = rows(k, cout)
        halo = ((R + 2) * k["kHaloW"] * 32 + 1023) // 1024 * 1024
        wts = (9 * npad * 32 + 1023) // 1024 * 1024
        # weights resident for the whole kernel when they fit, then the stages hold halos only
        wbytes = cin // 16 * 9 * npad * 32
        resident = wbytes <= k["kResidentMaxBytes"]
        wres = (wbytes + 1023) // 1024 * 1024 if resident else 0
        stage = halo if resident else halo + wts
        S = min(k["kMaxStages"], (SMEM_MAX - k["kTmaHeader"] - wres) // stage)
        assert S >= 2, (kind, cin, cout)
        smem = max(k["kTmaHeader"] + wres + S * stage, k["kTmaMinSmem"])
        assert wres % 1024 == 0 and wbytes < 1 << 20  # TMA destination alignment, transaction count
        assert smem <= SMEM_MAX and smem > SMEM_SM // 2  # one CTA per SM
        assert stage % 1024 == 0 and k["kTmaHeader"] % 1024 == 0  # swizzle-pattern alignment of every TMA destination
        # TMA boxes: halo 16 ch x 130 px x (R + 2) rows, weights 16 ch x npad rows x 9 taps
        assert k["kHaloW"] <= 256 and R + 2 <= 256 and npad <= 256 and wrows <= 256
        box_halo, box_w = 16 * k["kHaloW"] * (R + 2) * 2, 16 * npad * 9 * 2
        assert box_halo <= halo and box_w <= wts
        assert box_halo + box_w < 1 << 20  # mbarrier transaction count
        # A rows in 32-byte steps: the last tap of the last row stays in the halo tile
        assert ((R - 1 + 2) * k["kHaloW"] + 2) * 32 + k["kStrip"] * 32 <= (R + 2) * k["kHaloW"] * 32
        assert 8 * npad * 32 + npad * 32 <= wts
        # a resident chunk's nine taps at c * 9 * npad * 32, within the resident region
        assert not resident or (cin // 16) * 9 * npad * 32 <= wres
        # two accumulators and the bias table; nine mbarriers (full, empty x 4 stages, the
        # accumulators' pairs, the resident weights) before the TMEM address at byte 128
        assert 2 * R * npad <= 512 and 256 + 4 * npad <= k["kTmaHeader"]
        assert (2 * k["kMaxStages"] + 4 + 1) * 8 <= 128
        # every strip row has an issuing warp (rows r = m, m + MW, ...)
        assert k["kTmaMmaWarps"] >= 1 and 32 * (k["kTmaMmaWarps"] + 5) <= 1024


def test_channel_counts_fit_the_sixteen_channel_chunks(launches):
    """Both kernels step K 16 input channels at a time and read the decoder's two sources
    without a chunk straddling them: every input channel count and every coarse-level
    channel count is a multiple of 16."""
    for kind, cin, cout, wrows in launches:
        assert cin % 16 == 0
    # the decoder's inputs as forward() builds them: cat(coarse, cc, skip, cs)
    cats = re.findall(r"cat\(T_\w+, (\d+), T_\w+, (\d+)\)", _src("unet.cu"))
    assert len(cats) >= 4
    for cc, cs in cats:
        assert int(cc) % 16 == 0 and int(cs) % 8 == 0
