"""The persistent kernels' work order: static rounds, then items from a work
counter (take_item in xc_corr.cu).  Every pair must be processed exactly once
whatever CTA takes it, so a device batch and the same batch reversed (every
pair on another CTA and round) give each pair the same records, bit for bit,
and a sample of pairs run alone gives them too.  Batch sizes straddle
multiples of the one-CTA-per-SM grid, where the static rounds end (152 SMs on
GB300)."""
import numpy as np
import pytest

from satsuma2_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _per_pair(x, items):
    b = x.upload(items)
    b.run()
    res, counts = b.results(with_counts=True)
    b.free()
    out, o = [], 0
    for c in counts:
        out.append(res[o:o + int(c)].tobytes())
        o += int(c)
    return out


@pytest.mark.parametrize("n", [151, 152, 153, 304, 305, 457, 1217])
def test_pairs_processed_once_in_any_order(n):
    import satsuma2_gb300 as sg
    items = W.uniform_batch(n, seed=500 + n)
    x = sg.XCorr(target_total=4096.0 ** 2)
    fwd = _per_pair(x, items)
    rev = _per_pair(x, items[::-1])[::-1]
    assert fwd == rev
    for k in range(0, n, max(1, n // 6)):
        assert _per_pair(x, [items[k]])[0] == fwd[k], k
    assert sum(len(r) for r in fwd) > 0
    x.close()


def test_spectra_chunks_processed_once():
    """The spectra kernels' order: 13 x 17 pairs of 30 distinct chunks."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(7)
    ts = [W.random_bases(rng, 4096) for _ in range(17)]
    qs = [W.mutate(rng, t, 0.9, indel_every=0).tobytes() for t in ts[:13]]
    ts = [t.tobytes() for t in ts]
    items = [(t, q) for q in qs for t in ts]
    x = sg.XCorr(target_total=4096.0 * 17)
    b = x.upload(items)
    assert b.launches() == 6   # spectra, correlation from spectra, hand-back, scan, two finalize kernels
    b.free()
    fwd = _per_pair(x, items)
    rev = _per_pair(x, items[::-1])[::-1]
    assert fwd == rev
    assert sum(len(r) for r in fwd) > 0
    x.close()
