"""The tile autotuner (cgpu_autotune / cgpu_batch_autotune, cgpu_*_tiles).

* A batch of uneven trajectories in the 36-bit fixed-point form is tuned on
  its own shapes: the chosen table is the one applied, it is written to the
  cache, and a second batch of the same shapes takes it from the cache.
* Trajectories propagated with the tuned table and with the set-up
  heuristics' table agree to 1e-12 (the fixed-point contractions are exact
  digit sums whatever the tile; K splits and Lanczos blocks change FP64
  summation orders only).
* On one system every candidate table the tuner timed gives the same NonLin
  derivative (1e-12: the warm-started rho^-1 eigensolver carries ~1e-16
  differences from one evaluation to the next, which the double-float
  kernels, rounding at ~2^-44, can turn into ~1e-13; K-split partial sums
  round differently), and invalid tables are refused.
"""
import json

import numpy as np
import pytest

from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu


def _states(specs, systems, seed):
    out = []
    for k, (sp, s) in enumerate(zip(specs, systems)):
        rng = np.random.default_rng(seed + k)
        c = rng.normal(size=s.nC) + 1j * rng.normal(size=s.nC)
        out.append(I.pack_state(c / np.linalg.norm(c), I.seeded_gaussian_orbitals(sp, s.x, s.w, seed + k)))
    return out


def test_batch_autotune_applies_caches_and_keeps_results(tmp_path):
    from codyfortran_gb300.engine import Batch
    specs = S.batch_trajectory_specs(512, 1234)[:12]
    cache = tmp_path / "tiles.jsonl"
    a = Batch(specs, "mixed_fx6", max_krylov=12, krylov_window=1)
    states = _states(specs, a.systems, 40)
    a.upload(states)
    heuristic = a.tiles()
    rep = a.autotune(cache)
    assert rep["source"] == "tuned"
    chosen = {k: tuple(v) for k, v in rep["tiles"].items() if k != "lz_blocks"}
    chosen["lz_blocks"] = rep["tiles"]["lz_blocks"]
    assert a.tiles() == chosen
    for k in ("W", "Z", "H2"):
        cands = rep[f"{k}_candidates"]
        assert len(cands) >= 1 and all(c[3] > 0 for c in cands)
        best = min(cands, key=lambda c: c[3])
        assert tuple(best[:3]) == chosen[k]
    assert len(rep["lz_candidates"]) >= 2
    lines = [json.loads(l) for l in open(cache)]
    assert [l["key"] for l in lines] == [rep["key"]]
    # the same shapes again: the table comes from the cache
    b = Batch(specs, "mixed_fx6", max_krylov=12, krylov_window=1)
    b.upload(states)
    rep2 = b.autotune(cache)
    assert rep2["source"] == "cache" and rep2["key"] == rep["key"] and b.tiles() == chosen
    # tuned vs heuristic tables: same trajectories
    h = Batch(specs, "mixed_fx6", max_krylov=12, krylov_window=1)
    assert h.tiles() == heuristic
    h.upload(states)
    a.upload(states)
    a.propagate(0.0, 0.02, 5, 12)
    h.propagate(0.0, 0.02, 5, 12)
    ea, eh = a.energies(0.1), h.energies(0.1)
    assert np.max(np.abs(ea - eh) / np.abs(eh)) < 1e-12
    sa, sh = a.download_packed(), h.download_packed()
    assert np.linalg.norm(sa - sh) / np.linalg.norm(sh) < 1e-12
    for x in (a, b, h):
        x.close()


def test_every_timed_table_gives_the_same_derivative():
    from codyfortran_gb300.engine import CodyError, Engine
    sp = S.helium_fedvr(150, 6, 6, laser=S.sin2_pulse(0.05, omega=0.2, n_cycles=2.0))
    sp.xmin, sp.xmax = -150.0, 150.0
    e = Engine(sp, precision="mixed_fx6", max_krylov=12)
    st = _states([sp], [e], 3)[0]
    e.upload(st)
    ref = e.time_derivative(st, 1.0, "nonlin")
    rep = e.autotune(None, force=True)
    assert rep["source"] == "tuned"
    base = e.tiles()
    n_tables = 0
    errs = []
    for k in ("W", "Z", "H2"):
        for cand in rep[f"{k}_candidates"]:
            t = dict(base)
            t[k] = tuple(cand[:3])
            e.set_tiles(t)
            assert e.tiles()[k] == tuple(cand[:3])
            d = e.time_derivative(st, 1.0, "nonlin")
            errs.append((k, tuple(cand[:3]), float(np.linalg.norm(d - ref) / np.linalg.norm(ref))))
            n_tables += 1
    print("derivative deviation per table:", errs)
    # The contractions are exact sums, independent of the table.  What remains
    # is the rounding granularity of the form's double-float kernels (~2^-44)
    # under the ~1e-16 perturbations of the warm-started rho1 eigensolver,
    # which carries its eigenvectors from one evaluation to the next.
    assert max(err for _, _, err in errs) < 1e-12, errs
    assert n_tables >= 5
    for bad in ({**base, "W": (48, 0, 1)}, {**base, "lz_blocks": 0}, {**base, "Z": (base["Z"][0], 0, 999)}):
        with pytest.raises(CodyError):
            e.set_tiles(bad)
    e.close()
