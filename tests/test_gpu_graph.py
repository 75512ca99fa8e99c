"""CUDA-graph replay of the fused step (xdem_sim_set_graph) against eager
stepping: the same kernels with the same arguments in the same order, so the
state and the pair lists must be bit-identical, for odd and even step counts,
across a re-priming (set_state) and for both precision forms."""
import numpy as np
import pytest

from xdynamics_dll_gb300 import scenes, types as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def simmod():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, sim
    build.build()
    return sim


def _same(a, b):
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    for kind in range(3):
        for x, y in zip(a.pairs(kind), b.pairs(kind)):
            assert np.array_equal(x, y), kind


@pytest.mark.parametrize("precision", [T.XDEM_FP64, T.XDEM_MIXED])
def test_graph_replay_matches_eager(simmod, precision):
    sc = scenes.dam_break(n_target=6000)
    a = simmod.Sim(sc, precision=precision)
    b = simmod.Sim(sc, precision=precision)
    b.set_graph(True)
    for n in (1, 4, 3, 6):
        a.step(n)
        b.step(n)
        _same(a, b)
    # new state: both re-prime, the graph is captured again
    st = a.state()
    for s in (a, b):
        s.set_state(st["pos"], st["vel"], st["acc"], st["ep"], st["ev"], st["ea"], sc.mass, sc.inertia)
    a.step(5)
    b.step(5)
    _same(a, b)
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()


def test_mixed_fp32_copies_are_written_back_before_a_restart(simmod):
    """A mixed sphere handle keeps its accelerations in FP32 copies between
    steps and writes them back to the FP64 arrays before anything reads
    those.  Re-setting the pair lists makes the next step start over from the
    FP64 arrays (the first position update reads them): with a state read
    before it (write-back on the read) and without one (write-back inside the
    step) the runs stay bit-identical, graphs or not."""
    sc = scenes.dam_break(n_target=3000)
    hs = [simmod.Sim(sc, precision=T.XDEM_MIXED) for _ in range(3)]
    hs[2].set_graph(True)
    for h in hs:
        h.step(7)
    hs[0].state()
    for h in hs:
        for kind in range(2):
            cnt, ids, tsd = h.pairs(kind)
            h.set_pairs(kind, cnt, ids, tsd)
        h.step(9)
    _same(hs[0], hs[1])
    _same(hs[0], hs[2])
    for h in hs:
        assert h.status() == 0
        h.close()
