"""Autotuner search and cache logic (timing replaced by a model; no GPU)."""
import json

from gpumatfun_gb300 import autotune, workloads


def test_tune_picks_fastest_and_caches(tmp_path):
    P = workloads.config1_small(N=12, k=2, m=10, C=8, R=2)
    calls = []

    def fake(c):
        calls.append(c)
        return 1.0 + abs(c["threads"] - 256) / 256 + 0.5 * c["col_staging"] + 0.25 * c["sync_policy"] + 0.1 * c["blocks_per_sm"]

    path = tmp_path / "tune.json"
    r = autotune.tune(P, "mixed", cache_path=str(path), measure=fake)
    assert r["threads"] == 256 and r["col_staging"] == 1 and r["sync_policy"] == 0 and r["blocks_per_sm"] == 0
    assert not r["cached"] and r["trials"] == len(autotune.candidates(2)) == len(calls)
    r2 = autotune.tune(P, "mixed", cache_path=str(path), measure=fake)
    assert r2["cached"] and len(calls) == r["trials"]
    assert json.loads(path.read_text())[autotune.signature(P, "mixed")]["threads"] == 256
    # a different precision or workload is a different key
    assert autotune.signature(P, "fp64") != autotune.signature(P, "mixed")
    Q = workloads.config1_small(N=14, k=2, m=10, C=8, R=2)
    assert autotune.signature(Q, "mixed") != autotune.signature(P, "mixed")


def test_candidates_respect_rhs():
    assert all(c["blocks_per_sm"] in (0, 1) for c in autotune.candidates(4))
    assert {c["threads"] for c in autotune.candidates(1)} == {128, 256, 512}


def test_matrix_powers_candidates_only_with_a_polynomial():
    assert all(c["matrix_powers"] == 0 for c in autotune.candidates(1, 0))
    mp = [c for c in autotune.candidates(1, 8) if c["matrix_powers"] == 1]
    assert mp and all(c["sync_policy"] == 0 for c in mp)


def test_tune_batch_picks_fastest_and_caches(tmp_path):
    probs = workloads.config5_batch(nprob=4, R=4, seed=1, lo=10, hi=20, m=8, C=8)
    calls = []

    def fake(c):
        calls.append(c)
        return 2.0 - (c["threads"] == 512) - 0.5 * (c["blocks_per_sm"] == 1) + 0.3 * c["sync_policy"]

    path = tmp_path / "tune.json"
    r = autotune.tune_batch(probs, "mixed", cache_path=str(path), measure=fake)
    assert (r["threads"], r["blocks_per_sm"], r["sync_policy"]) == (512, 1, 0) and not r["cached"]
    assert r["trials"] == len(autotune.batch_candidates(4)) == len(calls)
    assert all(c["blocks_per_sm"] in (0, 1) for c in autotune.batch_candidates(4))
    r2 = autotune.tune_batch(probs, "mixed", cache_path=str(path), measure=fake)
    assert r2["cached"] and len(calls) == r["trials"]
    # the batch key differs from any single problem's and from another batch's
    assert autotune.batch_signature(probs, "mixed") != autotune.signature(probs[0], "mixed")
    assert autotune.batch_signature(probs[:3], "mixed") != autotune.batch_signature(probs, "mixed")


def test_sigma_candidates_only_for_ragged_rows():
    import numpy as np
    import scipy.sparse as sp
    P = workloads.config1_small(N=12, k=2, m=10, C=8, R=1)
    assert not autotune.ragged(P)                       # 5-point stencil: uniform rows
    assert all(c["sell_sigma"] == 0 for c in autotune.candidates(1, 0, autotune.ragged(P)))
    # one dense row in every 32 makes SELL-32 slices mostly padding
    n = 256
    rows, cols = [np.arange(n)], [np.arange(n)]
    for r in range(0, n, 32):
        rows.append(np.full(64, r)); cols.append(np.arange(64))
    A = sp.csr_matrix((np.ones(sum(len(x) for x in rows)), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    Q = workloads.make_problem("ragged", A + A.T, np.ones((n, 1)), np.zeros((n, 0)), np.zeros(0),
                               P.funcs[:1], 8, 8, 0.5, 200.0)
    assert autotune.ragged(Q)
    sig = [c for c in autotune.candidates(1, 4, True) if c["sell_sigma"]]
    assert sig and all(c["matrix_powers"] == 0 for c in sig)
