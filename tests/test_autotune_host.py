"""Host logic of the launch-shape autotuner: the sweep, the cache key, the cache file."""

import numpy as np

from traffic_assignment_gb300 import autotune as A
from traffic_assignment_gb300 import synth


def test_candidates_cover_every_variant_and_block():
    c = A.candidates()
    assert {x.sssp_variant for x in c} == {"rounds", "async", "nearfar", "nearfar_queue"}
    # (0: the library's choice for the precision and network size)
    assert {x.sssp_block for x in c} == {0, 128, 256, 512, 1024}
    assert {x.aon_block for x in c} == {0, 256, 512, 1024}
    assert len(set(c)) == len(c)
    q = A.candidates(quick=True)
    assert set(q) <= set(c)
    # small networks also try the edge-list sweeps; large ones do not
    small, _ = synth.make_grid416()
    big, _ = synth.make_grid10k()
    assert "small" in {x.sssp_variant for x in A.candidates(net=small)}
    assert "small" not in {x.sssp_variant for x in A.candidates(net=big)}


def test_solver_kwargs():
    net, _ = synth.make_small24()
    kw = A.Candidate("nearfar", 128, 8.0, 1024).solver_kwargs(net)
    assert kw["sssp_block"] == 128 and kw["aon_block"] == 1024
    assert kw["nf_delta"] == 8.0 * np.mean(net.fft)
    assert "nf_delta" not in A.Candidate("rounds", 512).solver_kwargs(net)


def test_cache_key_tracks_network_precision_batch_and_device():
    net, _ = synth.make_small24()
    k = A.cache_key(net, "fp32", 32, "GB300")
    assert k == A.cache_key(net, "fp32", 32, "GB300")
    assert k != A.cache_key(net, "fp64", 32, "GB300")
    assert k != A.cache_key(net, "fp32", 64, "GB300")
    assert k != A.cache_key(net, "fp32", 32, "other")
    net.capacity = net.capacity.copy()
    net.capacity[3] *= 2
    assert k != A.cache_key(net, "fp32", 32, "GB300")


def test_cache_round_trip(tmp_path):
    p = str(tmp_path / "tune.json")
    res = A.TuneResult(A.Candidate("async", 512), 1.25, [{"x": 1}], "k1")
    A._store_cache(p, "k1", res)
    A._store_cache(p, "k2", A.TuneResult(A.Candidate(), 2.0, [], "k2"))
    data = A._load_cache(p)
    assert set(data) == {"k1", "k2"}
    assert A.Candidate(**data["k1"]["best"]) == A.Candidate("async", 512)
    assert A._load_cache(str(tmp_path / "missing.json")) == {}
