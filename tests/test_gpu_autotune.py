"""The per-pair kernel's launch shape (kinc_sim_set_launch / kinc_sim_autotune): every shape gives
bit-identical results, the autotuner picks one of the timed candidates, and its cache answers a
second call without timing anything."""
import numpy as np
import pytest

from kinc_gb300 import Similarity, _native, synthetic

pytestmark = pytest.mark.gpu

# warps per CTA divide the kernel's warp count: 20 for GMM, 16 otherwise
SHAPES = {"gmm": [(20, 1, 8), (10, 1, 0), (4, 0, 16), (20, 0, 4)],
          "kmeans": [(16, 1, 8), (8, 1, 0), (4, 0, 16), (16, 0, 4)]}


@pytest.mark.parametrize("args", [dict(clusmethod="gmm", corrmethod="spearman", crit="BIC", preout=True,
                                       postout=True),
                                  dict(clusmethod="kmeans", corrmethod="pearson", maxclus=3, crit="BIC")],
                         ids=["gmm", "kmeans"])
def test_every_launch_shape_gives_the_same_bits(args):
    gem = synthetic.generate(2, genes=70, samples=150)
    sim = Similarity(gem, **args)
    sim.initialize()
    total = sim.total_pairs()
    want = None
    for w, r, p in SHAPES[args["clusmethod"]]:
        sim.set_launch(w, r, p)
        assert sim.launch() == {"warps_per_cta": w, "rounds": r, "prefetch": p}
        res = sim.execute(None, start=0, size=total)
        got = (res.K, res.labels[res.K > 1], np.nan_to_num(res.corr, nan=9.0).view(np.uint32))
        if want is None:
            want = got
        else:
            for a, b in zip(got, want):
                assert np.array_equal(a, b)
    sim.close()


def test_launch_shape_rejects_unsupported_values():
    gem = synthetic.generate(2, genes=20, samples=60)
    sim = Similarity(gem, clusmethod="gmm")
    sim.initialize()
    with pytest.raises(_native.SimError):
        sim.set_launch(5, 1, 8)
    with pytest.raises(_native.SimError):
        sim.set_launch(16, 1, 8)       # does not divide GMM's 20 warps
    with pytest.raises(_native.SimError):
        sim.set_launch(16, 2, 8)
    sim.close()


def test_autotune_picks_a_timed_candidate_and_caches_it(tmp_path, monkeypatch):
    monkeypatch.setenv("KINC_TUNE_CACHE", str(tmp_path / "launch.txt"))
    gem = synthetic.generate(2, genes=120, samples=200)
    sim = Similarity(gem, clusmethod="gmm", corrmethod="spearman", crit="BIC")
    sim.initialize()
    chosen, timed = sim.autotune(start=0, size=sim.total_pairs())
    assert len(timed) >= 4
    fastest = min(timed, key=lambda e: e["ms"])
    assert chosen == {k: fastest[k] for k in ("warps_per_cta", "rounds", "prefetch")}
    assert sim.launch() == chosen
    again, timed2 = sim.autotune(start=0, size=sim.total_pairs())
    assert again == chosen and timed2 == []
    assert (tmp_path / "launch.txt").read_text().count("\t") == 2
    sim.close()
