"""The request server: results of grids submitted in a mix (continuous
batching over several lanes) equal each grid's complex computed alone."""
import threading

import numpy as np
import pytest

from helpers import assert_same_complex, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu

KEYS = ("cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


def alone(M, f, tresh):
    r = full_rect(f)
    m = M.GridDataset(r, r).init(f).work().writeout_connectivity()
    if tresh > 0:
        m.simplify_un_simplify(tresh)
    return m.export()


def test_server_mix_equals_alone(gpu_lib):
    from mscomplex_gb300 import synth
    rng = np.random.default_rng(4)
    fields, tr = [], []
    for i in range(40):
        side = int(rng.integers(20, 300))
        f = synth.mixed_grid(side, 100 + i, quantize=256 if i % 10 == 0 else 0)
        fields.append(f)
        tr.append(float(rng.uniform(0, 0.05)) if i % 10 else 0.0)
    srv = gpu_lib.GridServer(arena_bytes=64 << 20, lanes=2, max_batch=8)
    ids = [srv.submit(f, t) for f, t in zip(fields, tr)]
    for rid, f, t in zip(ids, fields, tr):
        got = srv.result(rid)
        assert_same_complex(got, alone(gpu_lib, f, t), f"request {rid}", keys=KEYS)
        s, a, d = got["times_ms"]
        assert s <= a <= d
    st = srv.stats()
    assert st["grids_done"] == 40 and st["batches"] >= 2
    srv.close()


def test_server_concurrent_submitters(gpu_lib, oracle):
    srv = gpu_lib.GridServer(arena_bytes=1 << 30, lanes=3, max_batch=4)
    fields = [smooth_field(30 + 7 * i, 40 + 3 * i, i) for i in range(12)] + [tie_field(30, 35, 4, 2)]
    out = {}

    def client(lo, hi):
        for i in range(lo, hi):
            out[i] = srv.submit(fields[i], 0.05)

    th = [threading.Thread(target=client, args=(k * 5, min(len(fields), k * 5 + 5))) for k in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, f in enumerate(fields):
        r = full_rect(f)
        want = oracle.Dataset(f, r, r, tresh=0.05).msc()
        assert_same_complex(srv.result(out[i]), want, f"client grid {i}", keys=KEYS)
    srv.close()


def test_server_oversize_request_runs_alone(gpu_lib):
    srv = gpu_lib.GridServer(arena_bytes=1 << 16, lanes=1, max_batch=16)
    f = smooth_field(120, 100, 3)
    got = srv.result(srv.submit(f, 0.02))
    assert_same_complex(got, alone(gpu_lib, f, 0.02), "oversize", keys=KEYS)
    srv.close()


def test_server_bad_request(gpu_lib):
    srv = gpu_lib.GridServer(arena_bytes=1 << 20, lanes=1, max_batch=4)
    with pytest.raises(gpu_lib.DmscError):
        srv.submit(np.zeros((1, 4), np.float32))
    f = smooth_field(20, 20, 1).copy()
    f[2, 2] = np.nan
    rid = srv.submit(f)
    with pytest.raises(gpu_lib.DmscError):
        srv.result(rid)
    srv.close()


def test_server_budget_failure_fails_alone(gpu_lib):
    """A request that exhausts the simplification budget fails with its own
    error; the requests batched with it complete unchanged."""
    fields = [smooth_field(60, 60, 0), tie_field(40, 50, 5, 1), smooth_field(50, 70, 2), tie_field(20, 24, 5, 3)]
    tresh = [0.05, 0.3, 0.05, 0.3]
    full = gpu_lib.GridBatch().run(fields, tresh)
    ops = [full.simplify_stats(i)["ops"] for i in range(4)]
    budget = max(ops[0], ops[2], ops[3])
    assert ops[1] > budget, ops
    srv = gpu_lib.GridServer(arena_bytes=1 << 30, lanes=2, max_batch=8, max_ops=budget)
    ids = [srv.submit(f, t) for f, t in zip(fields, tresh)]
    for i, (rid, f, t) in enumerate(zip(ids, fields, tresh)):
        if i == 1:
            with pytest.raises(gpu_lib.DmscError) as ei:
                srv.result(rid)
            assert ei.value.code == 5
        else:
            assert_same_complex(srv.result(rid), alone(gpu_lib, f, t), f"request {i}", keys=KEYS)
    srv.close()
