"""Batched ensemble step: every run of a concatenated batch evolves exactly as it does
alone (bitwise: runs never interact and each keeps its own CFL time step), with
default and autotuned launch shapes, eagerly and through a CUDA graph."""
import numpy as np
import pytest
import torch

import phd_code_gb300 as pkg
from phd_code_gb300.autotune import tune
from phd_code_gb300.ensemble import EnsembleStepper, SequentialEnsemble
from phd_code_gb300.problems import riemann_ensemble

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def runs():
    r, _ = riemann_ensemble(n_runs=6, n_min=200, n_max=3000, seed=3)
    return r


def test_batch_equals_single_runs(runs):
    ens = EnsembleStepper(runs)
    ens.step(10)
    ens.check_status()
    for r, (m, p) in enumerate(runs):
        st = pkg.FluxStepper(m, p, precision="fp32", solver="hllc")
        st.step(10)
        assert np.array_equal(ens.run_cons(r), st.cons_host()[:, :m.n_real])
        assert ens.read_clocks()[r].dt == st.read_clock().dt


def test_graph_and_tuned_launch_are_bitwise_equal(runs):
    a = EnsembleStepper(runs)
    a.step(8)
    b = EnsembleStepper(runs)
    launch, table = tune(b, blocks=(128, 256), cap_waves=(0, 2), items=(1, 2, 4), reps=1)
    assert len(table) == 12
    assert (launch.items_grad, launch.items_face, launch.items_update) != (0, 0, 0)
    b.launch = launch
    b.capture(4)
    b.replay()
    b.replay()
    torch.cuda.synchronize()
    for r in range(len(runs)):
        assert np.array_equal(a.run_cons(r), b.run_cons(r))


@pytest.mark.parametrize("items", [1, 2, 4])
def test_every_tuned_shape_is_bitwise_equal(runs, items):
    """Each candidate of the tuner's space (block, grid cap, items per thread) advances
    the batch to the same bits as the default launch."""
    import phd_code_gb300._lib as L
    ref = EnsembleStepper(runs)
    ref.step(5)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for block in (128, 256, 512):
        for waves in (0, 2):
            e = EnsembleStepper(runs)
            cap = waves * sms
            e.launch = L.PhdLaunch(block, min(block, 256), block, cap, cap, cap, items, items, items)
            e.step(5)
            e.check_status()
            for r in range(len(runs)):
                assert np.array_equal(ref.run_cons(r), e.run_cons(r)), (block, waves, items, r)


def test_sequential_baseline_matches(runs):
    seq = SequentialEnsemble(runs)
    seq.step(3)
    ens = EnsembleStepper(runs)
    ens.step(3)
    for r, st in enumerate(seq.steppers):
        assert np.array_equal(ens.run_cons(r), st.cons_host()[:, :st.dmesh.n_real])
