"""The autotuner (xc_tune / xc_apply_tuning) and the kernel forms it chooses
between: the per-strand correlation kernel with 512, 256 or 128 threads per
strand, and at FFT 8192 the both-strands kernel forms or the per-strand
kernel alone.  Every form must give the same records bit for bit -- they run
the same butterflies and sums in the same order -- so each is checked against
the default context on a batch that spans FFT lengths 1024-8192 and holds
pairs the both-strands kernels hand back (N runs, ragged query lengths)."""
import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W
from tests import parity

pytestmark = pytest.mark.gpu


def _items():
    items = W.uneven_batch(160, seed=77)
    rng = np.random.default_rng(78)
    for k in range(8):
        t = W.random_bases(rng, 4096).tobytes()
        q = bytearray(t[300:3800] + W.random_bases(rng, 596).tobytes())
        if k % 2:
            q[1000:1100] = b"N" * 100
        else:
            q = q[:4096 - 5]
        items.append((t, bytes(q)))
    return items


def test_every_form_gives_the_default_records():
    import satsuma2_gb300 as sg
    items = _items()
    TT = float(sum(len(t) for t, _ in items))
    ref = sg.XCorr(fft_len=-1, target_total=TT)
    want = ref.align(items)
    assert len(want) > 100
    forms = ["fft_len=%d strand_threads=%d" % (L, nt) for L in (1024, 2048, 4096) for nt in (512, 256, 128)]
    forms += ["fft_len=8192 strand_threads=256", "fft_len=8192 pair_form=1",
              "fft_len=8192 pair_form=0 strand_threads=512", "fft_len=8192 pair_form=0 strand_threads=256"]
    for f in forms:
        x = sg.XCorr(fft_len=-1, target_total=TT)
        x.apply_tuning(f)
        got = x.align(items)
        assert parity.same_results(got, want, prob_rtol=0.0, target_total=0.0), f
        x.close()
    ref.close()


def test_tune_table_applies_and_keeps_results():
    import satsuma2_gb300 as sg
    items = _items()
    TT = float(sum(len(t) for t, _ in items))
    x = sg.XCorr(fft_len=-1, target_total=TT)
    want = x.align(items)
    table = x.tune()
    lines = [l for l in table.splitlines() if l.startswith("fft_len=")]
    assert [int(l.split()[0].split("=")[1]) for l in lines] == [1024, 2048, 4096, 8192], table
    assert all("corr_ms=" in l for l in lines)
    got = x.align(items)
    assert parity.same_results(got, want, prob_rtol=0.0, target_total=0.0)
    y = sg.XCorr(fft_len=-1, target_total=TT)
    y.apply_tuning(table)
    assert parity.same_results(y.align(items), want, prob_rtol=0.0, target_total=0.0)
    with pytest.raises(sg.XCError):
        y.apply_tuning("fft_len=16384 strand_threads=128")   # no such form
    y.close()
    x.close()


def test_small_strand_forms_vs_oracle():
    """The 128-thread form at FFT 1024-4096 against the oracle directly."""
    import satsuma2_gb300 as sg
    O = oracle.Oracle()
    items = [it for it in W.uneven_batch(300, seed=79) if W.uneven_fft_len(len(it[0]), len(it[1])) <= 4096][:24]
    TT = float(sum(len(t) for t, _ in items))
    x = sg.XCorr(fft_len=-1, target_total=TT)
    x.apply_tuning("fft_len=1024 strand_threads=128\nfft_len=2048 strand_threads=128\nfft_len=4096 strand_threads=128")
    res, counts = x.align(items, with_counts=True)
    o = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        d = x.debug_pair(t=t, q=q, signals=False)
        P = O.params(target_total=TT, fft_len=d["L"])
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=TT), k
    x.close()
