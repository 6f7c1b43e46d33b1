"""Serving: continuous batching of independent solves (ath_server_*).

Requests arrive while others run, are admitted as slots and device memory
allow, iterate concurrently on their own streams, retire on the device at the
residual drop, and hand back their final state.  Each result must equal the
result of the same solve run alone (bit for bit: the batches share no data
and every kernel is deterministic)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from aither_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _requests(tmp):
    from aither_gb300 import cases
    out = []
    specs = [(16, 8, 4, 0.06, 0.55), (20, 10, 3, 0.09, 0.75), (12, 12, 5, 0.04, 0.40),
             (24, 8, 4, 0.08, 0.65), (14, 10, 4, 0.05, 1.40)]
    for q, (ni, nj, nk, h, m) in enumerate(specs):
        inp, _ = cases.bump_channel(str(tmp / f"r{q}"), ni, nj, nk, h, m, name=f"r{q}")
        out.append(inp)
    pinp, _ = cases.flat_plate(str(tmp / "plate"), ni=10, nj=8, nk=2, dy0=1e-3, ratio=1.3,
                               name="plate")
    out.append(pinp)
    sinp, _ = cases.wall_channel(str(tmp / "sst"), 24, 12, 3, "bump", 0.08, 0.6, alpha=2.0,
                                 rans=True, stretch=1.1, name="sst")
    out.append(sinp)
    return out


def _alone(ctx, inp, precision, drop):
    from aither_gb300 import Batch, Setup
    s = Setup(inp)
    b = Batch(ctx, s, precision)
    info = b.converge(20000, drop, check_every=50)
    w = [b.field(k, "STATE") for k in range(s.counts()[1])]
    b.close()
    return info[0], w


def _serve(server, inps, gap_steps):
    """Submits the inputs one at a time, `gap_steps` scheduling passes apart,
    and runs the loop until every request has retired."""
    ids, done, max_active = [], {}, 0
    pending = list(inps)
    passes = 0
    while pending or len(done) < len(inps):
        if pending and passes % gap_steps == 0:
            ids.append(server.submit(pending.pop(0)))
        a, _ = server.step()
        max_active = max(max_active, a)
        for st in server.poll():
            done[st.id] = st
        passes += 1
        time.sleep(0.0005)
    return ids, done, max_active


@pytest.mark.parametrize("precision", [0, 1])
def test_served_results_equal_results_alone(ctx, precision, tmp_path):
    from aither_gb300 import Server
    inps = _requests(tmp_path)
    srv = Server(ctx, precision, drop=1e-4, max_iters=20000, chunk=37, max_active=8)
    ids, done, max_active = _serve(srv, inps, gap_steps=5)
    assert max_active >= 2  # requests overlapped on the device
    for rid, inp in zip(ids, inps):
        st = done[rid]
        info, w = _alone(ctx, inp, precision, 1e-4)
        assert st.converged == 1
        assert st.iterations == info.iterations
        for k, wk in enumerate(w):
            assert np.array_equal(srv.fetch(rid, k), wk)
        assert st.latency_ms >= st.queue_ms >= 0.0
        srv.release(rid)
    srv.close()


def test_admission_respects_the_memory_budget(tmp_path):
    """With a budget that holds one request at a time, requests queue and
    are admitted one by one as memory frees up; all complete."""
    from aither_gb300 import Context, Server
    inps = _requests(tmp_path)[:3]
    small = Context(0, hbm_budget=150 << 20)
    srv = Server(small, 0, drop=1e-3, max_iters=20000, chunk=50, max_active=8)
    ids, done, max_active = _serve(srv, inps, gap_steps=1)
    assert max_active == 1
    assert sorted(done) == sorted(ids)
    assert all(done[i].converged == 1 for i in ids)
    assert max(done[i].queue_ms for i in ids) > 0.0
    srv.close()
    small.close()
