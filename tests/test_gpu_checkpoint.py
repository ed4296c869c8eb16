"""Device checkpoints and the gather block-size autotuner (GPU)."""
import numpy as np
import pytest

from tests._support import gpu_domain
from weldform_gb300 import configs, PRECISION_MIXED

pytestmark = pytest.mark.gpu


def _state(d):
    return {f: d.get_array(f) for f in ("x", "v", "Sigma", "pl_strain", "Density")} | {"t": d.Time}


def test_checkpoint_rewinds_bit_exactly():
    d = gpu_domain()
    case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    d.prepare(case.dt)
    d.step(7)
    d.checkpoint_save(3)
    d.step(13)  # crosses neighbour rebuilds
    a = _state(d)
    d.checkpoint_restore(3)
    assert d.geti("steps") == 7
    d.step(13)
    b = _state(d)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    d.checkpoint_free(3)


def test_autotune_keeps_state_and_results():
    """The autotuner restores the state it timed from, and the run it leaves
    behind is bit-identical to one launched with its choice set directly (the
    block size never changes results; the lane count sets the gathers'
    summation order)."""
    res = []
    choice = None
    for tune in (True, False):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(3)
        if tune:
            before = _state(d)
            b = d.autotune(2)
            assert b in (64, 128, 256, 512)
            choice = (b, d.geti("gather_lanes"))
            assert choice[1] in (1, 2, 4, 8)
            after = _state(d)
            for k in before:
                assert np.array_equal(before[k], after[k]), k
        else:
            d.set("gather_lanes", choice[1])
        d.step(20)
        res.append(_state(d))
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k


@pytest.mark.gpu
def test_asynchronous_reads_snapshot_the_state_at_the_call():
    """wf_get_particle_array_f64_async: each read holds the field as it was
    when the read was enqueued, although steps run on while it copies, and
    more reads than the four snapshot buffers still all land (the fifth
    waits for the first).  Compared bit for bit with synchronous reads of an
    identical run."""
    torch = pytest.importorskip("torch")

    def run(asynchronous):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        n = d.particle_count
        out = []
        for k in range(6):
            d.step(3)
            if asynchronous:
                xo = torch.empty(n * 3, dtype=torch.float64).pin_memory().numpy()
                so = torch.empty(n * 9, dtype=torch.float64).pin_memory().numpy()
                out.append((d.get_array_async("x", xo), d.get_array_async("Sigma", so)))
            else:
                out.append((d.get_array("x").ravel().copy(), d.get_array("Sigma").ravel().copy()))
        if asynchronous:
            d.step(4)  # still running when the last reads are enqueued
            d.synchronize()
        out = [(x.copy(), s.copy()) for x, s in out]
        d.close()
        return out

    a, b = run(True), run(False)
    for (xa, sa), (xb, sb) in zip(a, b):
        assert np.array_equal(xa, xb) and np.array_equal(sa, sb)
    assert not np.array_equal(a[0][0], a[-1][0])


@pytest.mark.gpu
def test_conditional_search_graph_matches_the_gated_graph():
    """search_conditional: the step graph's search in a conditional node gives
    bit-identical results to the default gated form, through searches
    (yielding cylinder, a search every 5 steps)."""
    out = []
    for cond in (0, 1):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        d.set("search_conditional", cond)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(60)
        assert d.geti("search_conditional") == cond
        out.append((d.get_array("x"), d.get_array("Sigma"), d.geti("nb_searches")))
        d.close()
    assert out[0][2] == out[1][2] > 5
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
