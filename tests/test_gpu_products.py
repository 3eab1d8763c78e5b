"""Products of the sensor model that round to even and that underflow, on every product path.

The reference multiplies each particle's table factors in beam order in double precision
(RangeLib.h:533-555, 558-612); every product is rounded to nearest even.  These tables make
the chains hard: factors with 1-4 significant bits (a product drops only a few bits, so exact
ties come every few multiplies), and the same factors scaled by 2^-16 .. 2^-19 with some zeros
(61-beam products end as small normals, subnormals or zero).  The fused kernel under its tile
and beam-major schedules, eval_sensor_model, and the persistent batch with overlapped and
separate products must give the oracle's plain C doubles bit for bit.
"""
import numpy as np
import pytest

from range_libc_gb300 import workloads as W


def _tables(K, seed):
    """A table whose factors have 1-4 significant bits (products drop one to a few bits, so a
    tie to even comes every few multiplies), and one of such factors scaled by 2^-16 .. 2^-19
    with a few zeros (61-beam products end as small normals, subnormals or zero)."""
    rng = np.random.default_rng(seed)
    sig = 1.0 + rng.integers(0, 8, (K, K)) / 8.0
    ties = np.ldexp(sig, -rng.integers(0, 3, (K, K))).astype(np.float64)
    under = np.ldexp(sig, -rng.integers(16, 20, (K, K))).astype(np.float64)
    under[:, :3] = 0.0                  # a few zero factors
    return ties, under


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.gpu
@pytest.mark.parametrize("table_kind", ["ties", "underflow"])
def test_products_round_like_the_oracle(rl, oracle_mod, table_kind):
    torch = pytest.importorskip("torch")
    wl = W.particle_filter_step(side=512, n_particles=300, n_beams=61, max_range_px=200.0, seed=2024,
                                origin=(-1.25, -2.5))
    K = wl.table.shape[0]
    table = _tables(K, 5)[0 if table_kind == "ties" else 1]
    m = rl.PyOMap(np.ascontiguousarray(wl.occ.T))
    m.set_world(*wl.world[:4])
    g = rl.PyRayMarchingGPU(m, wl.max_range)
    ref = oracle_mod.OracleMethod(wl.occ, "rm", wl.max_range, world=m.world)
    g.set_sensor_model(table)
    ref.set_sensor_model(table)
    _, trig = oracle_mod.world_rays(m.world, wl.ins, wl.angles)
    g.set_trig_override(trig)
    n, na = len(wl.ins), len(wl.angles)
    exp_w = ref.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs)
    if table_kind == "underflow":
        tiny = np.finfo(np.float64).tiny
        assert (exp_w == 0).any() and ((exp_w > 0) & (exp_w < tiny)).any() and (exp_w >= tiny).any()
    else:
        assert np.all(exp_w > 0)
    w = np.empty(n, np.float64)
    for sched in ((0, 128, 0, 0), (4, 256, 0, 8), (5, 512, 0, 32), (3, 0, 0, 0)):
        g.set_schedule(*sched)
        w[:] = -1.0
        g.calc_range_repeat_angles_eval_sensor_model(wl.ins, wl.angles, wl.obs, w)
        assert np.array_equal(_bits(w), _bits(exp_w)), sched
    # eval_sensor_model on the oracle's own ranges
    ranges = ref.calc_range_repeat_angles(wl.ins, wl.angles)
    w[:] = -1.0
    g.eval_sensor_model(wl.obs, ranges, w, na, n)
    assert np.array_equal(_bits(w), _bits(ref.eval_sensor_model(wl.obs, ranges, na, n)))
    # the persistent batch, products overlapped and in a second launch
    dev = torch.device("cuda:0")
    t = [torch.from_numpy(a).to(dev) for a in (wl.ins, wl.angles, wl.obs)]
    tw = torch.zeros(n, dtype=torch.float64, device=dev)
    batch = rl.PyFilterBatch([(g, t[0], t[1], t[2], tw)])
    for separate in (False, True):
        batch.set_product_mode(separate)
        tw.fill_(-1.0)
        batch.run()
        torch.cuda.synchronize()
        assert np.array_equal(_bits(tw.cpu().numpy()), _bits(exp_w)), separate
