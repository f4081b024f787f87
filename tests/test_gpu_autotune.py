"""The batch launch autotuner (dmsc_batch_autotune; no reference
counterpart): it picks, per size class, the threads per block and resident
blocks per SM of the two persistent tile kernels.  The complexes must not
depend on the configuration: every configuration, the tuned one and the
untuned single launch give the same bytes, and those equal the oracle's."""
import numpy as np
import pytest

from helpers import assert_same_complex, full_rect

pytestmark = pytest.mark.gpu

KEYS = ("rect_ext", "cellid", "fn", "pair_idx", "flags", "asc_off", "asc", "des_off", "des")


def sample():
    from mscomplex_gb300 import synth
    # one or two grids of each class below 1024, and one above
    sides = [64, 100, 180, 250, 300, 700, 1100]
    return [synth.mixed_grid(s, 7001 + i) for i, s in enumerate(sides)]


def exports(M, ctx, fields, tresh):
    b = M.GridBatch(ctx).run(fields, tresh)
    return [b.export(i) for i in range(len(fields))]


def test_autotune_table_and_unchanged_results(gpu_lib, oracle):
    fields = sample()
    ctx = gpu_lib.Context()
    base = exports(gpu_lib, ctx, fields, 0.02)
    for i, f in enumerate(fields):
        r = full_rect(f)
        assert_same_complex(base[i], oracle.Dataset(f, r, r, tresh=0.02).msc(), f"untuned grid {i}", keys=KEYS)
    table = gpu_lib.GridBatch.autotune(fields, repeats=2, ctx=ctx)
    assert set(table) == {"<128", "<256", "<512", "<1024", "<2048"}
    for cls, (threads, bps, us, default_us) in table.items():
        assert threads in (256, 512) and 1 <= bps <= 3, (cls, threads, bps)
        assert 0 < us <= default_us, (cls, us, default_us)
    tuned = exports(gpu_lib, ctx, fields, 0.02)
    for i in range(len(fields)):
        assert_same_complex(tuned[i], base[i], f"tuned grid {i}", keys=KEYS)
    ctx.close()


@pytest.mark.parametrize("threads,bps", [(256, 1), (256, 3), (512, 1), (512, 2)])
def test_every_launch_configuration_gives_the_same_complexes(gpu_lib, threads, bps):
    fields = sample()
    ctx = gpu_lib.Context()
    base = exports(gpu_lib, ctx, fields, 0.02)
    for c in range(6):
        gpu_lib.GridBatch.set_launch(c, threads, bps, ctx=ctx)
    got = exports(gpu_lib, ctx, fields, 0.02)
    for i in range(len(fields)):
        assert_same_complex(got[i], base[i], f"{threads} threads x {bps} per SM, grid {i}", keys=KEYS)
    gpu_lib.GridBatch.autotune_reset(ctx=ctx)
    again = exports(gpu_lib, ctx, fields, 0.02)
    for i in range(len(fields)):
        assert_same_complex(again[i], base[i], f"after reset, grid {i}", keys=KEYS)
    ctx.close()


def test_launch_settings_rejected(gpu_lib):
    ctx = gpu_lib.Context()
    for args in ((6, 512, 3), (0, 384, 3), (0, 512, 0), (0, 512, 4)):
        with pytest.raises(gpu_lib.DmscError):
            gpu_lib.GridBatch.set_launch(*args, ctx=ctx)
    ctx.close()
