"""GPU parity of batches of whole grids (one shared pass of work +
writeout_connectivity + simplify_un_simplify over grids of different sizes)
against the oracle's single-grid path (dmsc/src/grid_dataset.cpp:1734-1907,
dmsc/src/grid_mscomplex.cpp:384-535), grid by grid."""
import numpy as np
import pytest

from helpers import assert_same_complex, full_rect, smooth_field, tie_field

pytestmark = pytest.mark.gpu

KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


def check_batch(M, oracle, fields, tresh, what):
    b = M.GridBatch().run(fields, tresh)
    t = np.broadcast_to(np.asarray(tresh, np.float64), (len(fields),))
    for i, f in enumerate(fields):
        r = full_rect(f)
        want = oracle.Dataset(f, r, r, tresh=float(t[i])).msc()
        assert_same_complex(b.export(i), want, f"{what} grid {i} {f.shape} t={t[i]}", keys=KEYS)
    return b


def test_batch_shapes(gpu_lib, oracle):
    fields = [smooth_field(2, 2, 0), smooth_field(3, 7, 1), smooth_field(65, 64, 2), smooth_field(64, 65, 3),
              smooth_field(130, 70, 4), smooth_field(9, 200, 5)]
    check_batch(gpu_lib, oracle, fields, 0.0, "shapes")


def test_batch_simplified_mixed_thresholds(gpu_lib, oracle):
    fields = [smooth_field(70, 90, s) for s in range(4)] + [tie_field(40, 50, 5, s) for s in range(3)]
    tresh = [0.0, 0.05, 0.3, 0.01, 0.3, 0.0, 0.3]
    check_batch(gpu_lib, oracle, fields, tresh, "mixed")


def test_batch_mixed_grids(gpu_lib, oracle):
    from mscomplex_gb300 import synth
    fields = synth.batch_fields(count=12, seed=3, lo=16, hi=300)
    check_batch(gpu_lib, oracle, fields, 0.02, "batch_fields")


def test_batch_matches_single_grid_path(gpu_lib):
    from mscomplex_gb300 import synth
    fields = synth.batch_fields(count=6, seed=7, lo=64, hi=700)
    b = gpu_lib.GridBatch().run(fields, 0.02)
    for i, f in enumerate(fields):
        r = full_rect(f)
        m = gpu_lib.GridDataset(r, r).init(f).work().writeout_connectivity()
        m.simplify_un_simplify(0.02)
        one = m.export()
        assert_same_complex(b.export(i), one, f"single vs batch grid {i}", keys=KEYS)
        assert b.simplify_stats(i) == m.simplify_stats()


def test_batch_rerun_in_place_and_export_all(gpu_lib, oracle):
    b = gpu_lib.GridBatch()
    f1 = [smooth_field(50, 60, s) for s in range(3)]
    b.run(f1, 0.05)
    f2 = [tie_field(30, 20, 4, 1), smooth_field(200, 150, 9)]
    b.run(f2, [0.3, 0.02])
    assert b.n == 2
    allx = b.export_all()
    for i, f in enumerate(f2):
        r = full_rect(f)
        want = oracle.Dataset(f, r, r, tresh=[0.3, 0.02][i]).msc()
        got = b.export(i)
        assert_same_complex(got, want, f"rerun grid {i}", keys=KEYS)
        c0, c1 = allx["cp_base"][i], allx["cp_base"][i + 1]
        a0, d0 = allx["asc_base"][i], allx["des_base"][i]
        assert np.array_equal(allx["cellid"][c0:c1].view(np.int16).reshape(-1, 2), got["cellid"])
        assert np.array_equal(allx["asc_off"][c0:c1 + 1] - a0, got["asc_off"])
        assert np.array_equal(allx["des_off"][c0:c1 + 1] - d0, got["des_off"])
        assert np.array_equal(allx["asc"][a0:allx["asc_base"][i + 1]], got["asc"])


def test_batch_device_input(gpu_lib, oracle):
    import torch
    fields = [smooth_field(40, 33, 1), smooth_field(90, 64, 2)]
    packed, sizes = gpu_lib.GridBatch.pack(fields)
    b = gpu_lib.GridBatch().run(packed=torch.from_numpy(packed).cuda(), sizes=sizes, tresh=0.05)
    for i, f in enumerate(fields):
        r = full_rect(f)
        assert_same_complex(b.export(i), oracle.Dataset(f, r, r, tresh=0.05).msc(), f"device grid {i}", keys=KEYS)


def test_batch_bad_input(gpu_lib):
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridBatch().run([np.zeros((1, 5), np.float32)])
    f = smooth_field(20, 20, 1).copy()
    f[3, 4] = np.nan
    with pytest.raises(gpu_lib.DmscError):
        gpu_lib.GridBatch().run([smooth_field(10, 10, 0), f])


def budget_case(M):
    """Three grids whose middle one (exact ties everywhere) needs more
    simplification operations than the other two; the budget is the largest
    of the other two's counts."""
    fields = [smooth_field(60, 60, 0), tie_field(40, 50, 5, 1), smooth_field(50, 70, 2)]
    tresh = [0.05, 0.3, 0.05]
    full = M.GridBatch().run(fields, tresh)
    ops = [full.simplify_stats(i)["ops"] for i in range(3)]
    assert ops[1] > max(ops[0], ops[2]), ops
    return fields, tresh, max(ops[0], ops[2])


def test_batch_budget_failure_is_per_grid(gpu_lib, oracle):
    fields, tresh, budget = budget_case(gpu_lib)
    with pytest.raises(gpu_lib.DmscError) as ei:
        gpu_lib.GridBatch().run(fields, tresh, max_ops=budget)
    assert ei.value.code == 9  # DMSC_ERR_PARTIAL
    b = gpu_lib.GridBatch().run(fields, tresh, max_ops=budget, partial_ok=True)
    code, msg = b.grid_status(1)
    assert code == 5 and "budget" in msg  # DMSC_ERR_DEVICE_TIMEOUT
    for i in (0, 2):
        assert b.grid_status(i) == (0, "")
        r = full_rect(fields[i])
        want = oracle.Dataset(fields[i], r, r, tresh=tresh[i]).msc()
        assert_same_complex(b.export(i), want, f"budget batch grid {i}", keys=KEYS)
    with pytest.raises(gpu_lib.DmscError) as ei:
        b.export(1)
    assert ei.value.code == 5
    with pytest.raises(gpu_lib.DmscError):
        b.export_all()


def test_batch_largest_mixed_grids_vs_oracle(gpu_lib, oracle):
    """The mixed-size workload's largest grids (sides 2034-2046, and two near
    1024), generated as the batch workload generates them, in one batch with
    small grids, each against the oracle at 2% of its range."""
    from mscomplex_gb300 import synth
    sides = synth.mixed_batch_sides(1000, 3)
    order = np.argsort(-sides)
    near_1k = np.argsort(np.abs(sides - 1024))[:2]
    pick = [int(i) for i in order[:4]] + [int(i) for i in near_1k] + [int(i) for i in order[-3:]]
    fields = [synth.mixed_grid(int(sides[i]), 3 * 1000003 + i) for i in pick]
    check_batch(gpu_lib, oracle, fields, 0.02, "largest mixed grids")
