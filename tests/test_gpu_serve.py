"""GPU: the serving loop (yaksa_gb300_serve_trace) replays a Poisson arrival schedule
through the plain nonblocking path and through the persistent server; every request
gives the oracle's bytes in both, alone (one request per trace) and in the mix, and
latencies are non-negative with the makespan covering the last arrival.

Tolerance: byte-identical (REPLACE and integer operators; the float operators are
elementwise in the same order as the oracle, and no input here produces NaN).
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import assert_same_bytes, host_of
from test_gpu_server import make_requests, op_of, oracle_apply

pytestmark = pytest.mark.gpu


def reset(cuda, reqs):
    for r in reqs:
        r["t_g"].copy_(cuda.from_numpy(r["typed"]))
        r["p_g"].copy_(cuda.from_numpy(r["packed"]))
    cuda.cuda.synchronize()


def check(cuda, oracle, reqs, ops):
    for i, r in enumerate(reqs):
        th, ph, a = oracle_apply(oracle, r)
        assert ops[i].actual == a
        assert_same_bytes(host_of(cuda, r["t_g"]), th, f"request {i} typed", r["base"])
        assert_same_bytes(host_of(cuda, r["p_g"]), ph, f"request {i} packed", r["base"])


@pytest.mark.parametrize("mode", ["plain", "server"])
@pytest.mark.parametrize("seed", range(2))
def test_serve_trace_matches_oracle(cuda, prod, oracle, mode, seed):
    g, reqs = make_requests(cuda, prod, oracle, 500 + seed, 60)
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1 / 20e3, len(reqs)))
    arrivals -= arrivals[0]
    srv = yk.Server(prod, ring_requests=16, budget_bytes=1 << 20) if mode == "server" else None
    ops = prod.batch_array([op_of(r) for r in reqs])
    lat, mk = yk.serve_trace(prod, ops, arrivals.tolist(), server=srv)
    cuda.cuda.synchronize()
    assert all(x >= 0 for x in lat)
    assert mk >= arrivals[-1]
    check(cuda, oracle, reqs, ops)
    # alone: each request in a trace of its own gives the same bytes
    reset(cuda, reqs)
    for i in range(len(reqs)):
        one = prod.batch_array([op_of(reqs[i])])
        yk.serve_trace(prod, one, [0.0], server=srv)
    cuda.cuda.synchronize()
    check(cuda, oracle, reqs, ops)
    if srv:
        srv.destroy()
    for r in reqs:
        r["pair"].free()
    g.free()


def test_serve_trace_empty(prod):
    lat, mk = yk.serve_trace(prod, prod.batch_array([yk.pack_op(0, 0, yk.TYPE_INT32_T, 0, 0, 0)]),
                             [0.0])
    assert lat[0] >= 0 and mk >= 0


def test_graph_lane_replays_repeated_requests(cuda, prod, oracle):
    """mode 2: each of 30 REPLACE records arrives six times; every record is captured
    once (at its second sight) and replayed from then on, and the bytes equal the
    oracle's (a REPLACE repeated with the same inputs writes the same bytes)"""
    g, reqs = make_requests(cuda, prod, oracle, 700, 30, ops=False)
    reps = 6
    order = [i for _ in range(reps) for i in range(len(reqs))]
    ops = prod.batch_array([op_of(reqs[i]) for i in order])
    arrivals = np.linspace(0.0, 3e-3, len(order))
    s0 = prod.graph_lane_stats()
    lat, mk = yk.serve_trace(prod, ops, arrivals.tolist(), graphs=True)
    cuda.cuda.synchronize()
    s1 = prod.graph_lane_stats()
    moving = sum(1 for i in range(len(reqs)) if ops[i].actual > 0)
    assert moving > 20
    assert s1["captures"] - s0["captures"] == moving
    assert s1["replays"] - s0["replays"] == moving * (reps - 1)
    assert all(x >= 0 for x in lat) and mk >= arrivals[-1]
    for k in range(reps):
        for i in range(len(reqs)):
            assert ops[k * len(reqs) + i].actual == ops[i].actual
    check(cuda, oracle, reqs, ops)
    for r in reqs:
        r["pair"].free()
    g.free()
