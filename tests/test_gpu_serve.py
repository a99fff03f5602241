"""The serving form (f3d_server_*): requests that arrive while others run
are admitted as memory frees up, their work overlaps on the device, and each
result is the same as running that request alone (bit for bit: the batch
never mixes the arithmetic of two scenarios; the outflow budget agrees to a
few ulp, see test_gpu_batch)."""
import numpy as np
import pytest

import fall3d_gb300 as F
from fall3d_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL_BUDGET = 1e-14


def _requests():
    return [
        synth.make_scenario("small", seed=31, run_h=0.5),
        synth.make_scenario("small", seed=32, nx=44, ny=30, nz=12, nc=5, run_h=0.6, wetdep=True, M0=3e6),
        synth.make_scenario("tiny", seed=33, nx=25, ny=20, nz=10, nc=3, run_h=0.3),  # an odd nx
        synth.make_scenario("small", seed=34, nx=30, ny=36, nz=16, nc=4, run_h=0.4, H=6000.0),
    ]


def _alone(s):
    g = F.Context(s, F.PREC_FP32)
    log = g.run()
    out = g.outputs()
    g.close()
    return out, log


@pytest.fixture(scope="module")
def alone():
    return [_alone(s) for s in _requests()]


def _same(res, ref, tag):
    out, log = ref
    for k in ("load", "col_mass", "c_grnd"):
        assert np.array_equal(res[k], out[k]), (tag, k)
    lg = res["log"]
    assert np.array_equal(lg["iiter"], log["iiter"]), tag
    for k in ("massvol", "massdep", "massdry", "masswet", "erumass"):
        assert np.array_equal(lg[k], log[k]), (tag, k)
    scale = max(1.0, float(np.max(np.abs(log["outmass"]))))
    assert np.max(np.abs(lg["outmass"] - log["outmass"])) <= RTOL_BUDGET * scale, tag


def test_serving_alone_equals_in_mix(alone):
    reqs = _requests()
    fp = [F.Context.footprint(s, F.PREC_FP32) for s in reqs]
    # room for the first two only: the third waits until one of them ends
    srv = F.Server(fp[0] + fp[1] + 1, max_running=8)
    ids = [srv.submit(reqs[0]), srv.submit(reqs[1])]
    for _ in range(4):
        srv.progress(1)
    ids.append(srv.submit(reqs[2]))  # arrives while the first two run
    srv.progress(1)
    assert srv.poll(ids[2])["state"] == F.Server.QUEUED
    ids.append(srv.submit(reqs[3]))
    while True:
        running, queued = srv.progress(4)
        if running == 0 and queued == 0:
            break
    polls = [srv.poll(i) for i in ids]
    assert all(p["state"] == F.Server.DONE for p in polls), polls
    # the third request waited for memory: admitted only once an earlier one ended
    assert polls[2]["t_admit"] >= min(polls[0]["t_done"], polls[1]["t_done"])
    for i, rid in enumerate(ids):
        _same(srv.result(rid), alone[i], f"request {i}")
    st = srv.stats()
    assert st["used_bytes"] == 0 and st["running"] == 0
    srv.close()


def test_serving_rejects_request_larger_than_cap():
    s = synth.make_scenario("tiny", seed=1)
    srv = F.Server(1024, max_running=2)
    rid = srv.submit(s)
    srv.progress(1)
    p = srv.poll(rid)
    assert p["state"] == F.Server.FAILED and "cap" in p["error"]
    srv.close()
