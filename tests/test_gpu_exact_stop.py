"""The mixed-precision solve stops at the same sweep as the FP64 solve: its
coarse loop checks the norm every inner_sweeps sweeps, and when it stops
between two checks the last outer iteration is redone sweep by sweep (in
graph and eager execution, alone and in a batch)."""
import numpy as np
import pytest

from stroemung_gb300 import _lib, presets
from stroemung_gb300.batch import Batch
from stroemung_gb300.simulation import ARITH_FAST, PREC_FP64, PREC_MIXED, Simulation

pytestmark = pytest.mark.gpu


def _sim(precision, eps, execution=_lib.EXEC_GRAPH, itermax=600):
    return Simulation(grid=presets.cavity(64), cell_size=(1 / 64, 1 / 64), delt=1e-3, gamma=0.9,
                      reynolds=100.0, sor_absolute_epsilon=eps, max_iterations=itermax,
                      omega=1.7, tau=0.5, precision=precision, arithmetic=ARITH_FAST,
                      strict_eps=_lib.STOP_STRICT, execution=execution)


def _eps():
    """eps whose strict rule stops the first FP64 step after 150 sweeps or so."""
    probe = _sim(PREC_FP64, 1e-12)
    probe.run_simulation_tick()
    h = probe.residual_history()
    probe.close()
    return float(np.sqrt(h[h[:, 0] <= 150][-1, 1] * 1.0001))


@pytest.mark.parametrize("execution", [_lib.EXEC_GRAPH, _lib.EXEC_EAGER])
def test_mixed_stops_at_the_fp64_sweep(execution):
    eps = _eps()
    ref = _sim(PREC_FP64, eps)
    mix = _sim(PREC_MIXED, eps, execution)
    its_ref, its_mix = [], []
    for _ in range(6):
        its_ref.append(ref.run_simulation_tick()[0])
        its_mix.append(mix.run_simulation_tick()[0])
    assert its_mix == its_ref
    assert any(k % 16 for k in its_ref), its_ref  # stops between coarse checks happen
    h = mix.residual_history()
    assert int(h[-1, 0]) == its_mix[-1]
    for n in ("u", "v", "p"):
        a, b = mix.download(n), ref.download(n)
        if n == "p":
            a, b = a - a.mean(), b - b.mean()
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), n
    ref.close()
    mix.close()


def test_remaining_sweeps_when_max_iterations_is_not_a_multiple():
    ref = _sim(PREC_FP64, 1e-30, itermax=70)
    mix = _sim(PREC_MIXED, 1e-30, itermax=70)
    for _ in range(2):
        assert ref.run_simulation_tick()[0] == 70
        assert mix.run_simulation_tick()[0] == 70
    ref.close()
    mix.close()


def test_batch_member_redo_matches_single_run():
    eps = _eps()
    alone = _sim(PREC_MIXED, eps)
    its = [alone.run_simulation_tick()[0] for _ in range(4)]
    p_alone = alone.download("p")
    alone.close()
    member = _sim(PREC_MIXED, eps)
    member.set_mode(precision=PREC_MIXED, arithmetic=ARITH_FAST, strict_eps=_lib.STOP_STRICT,
                    sweep_schedule=3)
    other = Simulation(grid=presets.channel(128, 32), cell_size=(0.01, 0.01), delt=0.002,
                       gamma=0.9, reynolds=100.0, max_iterations=200, tau=0.5,
                       precision=PREC_MIXED, sweep_schedule=3)
    ref2 = _sim(PREC_MIXED, eps)
    ref2.set_mode(precision=PREC_MIXED, arithmetic=ARITH_FAST, strict_eps=_lib.STOP_STRICT,
                  sweep_schedule=3)
    its2 = [ref2.run_simulation_tick()[0] for _ in range(4)]
    with Batch([member, other]) as batch:
        st = batch.step(4)
    assert [int(x) for x in st[0]["sor_iterations"]] == its2 == its
    np.testing.assert_array_equal(member.download("p"), ref2.download("p"))
    for s in (member, other, ref2):
        s.close()
