"""Host logic of compiled families and parameter scans (compiled_families.jl, scans.jl);
no GPU: builders that fail before compilation exercise the failure policies."""
import numpy as np
import pytest

import picuda
from picuda.scans import _family_model, _family_rates


def _model():
    s = picuda.spin_matrices(2)
    return picuda.qubit_ensemble_model(6, hamiltonian=s["jx"], emission=0.3, dephasing=0.1,
                                       collective_emission=0.05)


def test_family_rate_selection_and_binding():
    """compiled_families.jl:53-64, 176-193, 78-85."""
    m = _model()
    fam = picuda.compile_family(m, rate_indices=[2, 0])
    assert fam.rate_indices == (0, 2)
    assert fam.default_rates == (m.terms[0].rate, m.terms[2].rate)
    assert _family_rates(fam, (1.5, 0.25)) == (1.5, 0.25)
    with pytest.raises(picuda.PiArgumentError):
        _family_rates(fam, 2.0)  # scalar needs exactly one selected rate
    with pytest.raises(picuda.PiDimensionMismatch):
        _family_rates(fam, (1.0, 2.0, 3.0))
    with pytest.raises(picuda.PiArgumentError):
        _family_rates(fam, (1.0, float("nan")))
    bound = _family_model(fam, (1.5, 0.25))
    assert bound.terms[0].rate == 1.5 and bound.terms[2].rate == 0.25
    assert bound.terms[1].rate == m.terms[1].rate and m.terms[0].rate != 1.5
    one = picuda.compile_family(m, rate_indices=[1])
    assert _family_rates(one, 0.7) == (0.7,)
    for bad in ([], [0, 0], [7], [True]):
        with pytest.raises((picuda.PiArgumentError, IndexError)):
            picuda.compile_family(m, rate_indices=bad)


def test_scan_plan_validation():
    """scans.jl:85-156 argument checks."""
    build = lambda p: _model()
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([], build)
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, task="dynamics")
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, solver_options={"initial_state": None})
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, seed=-1)
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], lambda a, b, c: None)
    plan = picuda.ParameterScanPlan([1.0, 2.0], build, continuation=True)
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, execution="batched")  # threaded execution requires continuation=false
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, on_error="ignore")
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, indices=[1, 0])
    with pytest.raises(IndexError):
        picuda.parameter_scan(plan, indices=[5])
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, max_points=-1)


def test_scan_failure_policies_and_callback():
    """on_error :stop / :record / :throw and the callback's :stop (scans.jl:1096-1131); the
    builder fails before any GPU work."""
    def build(p, index):
        raise picuda.PiArgumentError(f"bad point {index}")
    plan = picuda.ParameterScanPlan([0.1, 0.2, 0.3], build, continuation=False)
    stop = picuda.parameter_scan(plan)
    assert len(stop) == 1 and stop[0].status == "failed" and stop[0].error_type == "PiArgumentError"
    assert stop[0].message == "bad point 0" and not stop[0].converged
    rec = picuda.parameter_scan(plan, on_error="record")
    assert [p.index for p in rec] == [0, 1, 2] and all(p.status == "failed" for p in rec)
    assert rec.restart_index == 0
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, on_error="throw")
    seen = []
    cb = picuda.parameter_scan(plan, on_error="record", callback=lambda pt: (seen.append(pt.index), "stop")[1])
    assert len(cb) == 1 and seen == [0]
    sub = picuda.parameter_scan(plan, on_error="record", indices=[0, 2], max_points=1)
    assert [p.index for p in sub] == [0]
    with pytest.raises(picuda.PiArgumentError):
        picuda.parameter_scan(plan, on_error="record", callback=lambda pt: "continue")
    for ex in ("threads", "batched"):
        r = picuda.parameter_scan(plan, execution=ex, on_error="record")
        assert [p.status for p in r] == ["failed"] * 3


def test_spectral_scan_plan_validation():
    """scans.jl:93-102, 126-151 for task=:spectrum."""
    build = lambda p: _model()
    plan = picuda.ParameterScanPlan([1.0], build, task="spectrum", nev=3, solver_options={"krylovdim": 30})
    assert plan.task == "spectrum" and plan.nev == 3 and plan.solver_options == {"krylovdim": 30}
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, task="spectrum", nev=0)
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, task="spectrum", spectrum_target="smallest")
    # automatic selection near zero is harmonic Arnoldi (highlevel.jl:735-746); its Krylov
    # options move from solver_options into the algorithm record
    near = picuda.ParameterScanPlan([1.0], build, task="spectrum", spectrum_target="near_zero", nev=2,
                                    solver_options={"krylovdim": 12, "maxrestarts": 5, "require_convergence": False})
    assert near.algorithm == picuda.HarmonicArnoldiAlgorithm(nev=2, krylovdim=12, maxrestarts=5)
    assert near.solver_options == {"require_convergence": False}
    explicit = picuda.HarmonicArnoldiAlgorithm(nev=2, krylovdim=4, thickdim=2, maxrestarts=4)
    assert picuda.ParameterScanPlan([1.0], build, task="spectrum", algorithm=explicit).algorithm is explicit
    assert picuda.ParameterScanPlan([1.0], build, task="spectrum", algorithm="harmonic",
                                    nev=3).algorithm == picuda.HarmonicArnoldiAlgorithm(nev=3)
    assert picuda.ParameterScanPlan([1.0], build, task="spectrum", spectrum_target="near_zero",
                                    algorithm="arnoldi").algorithm == "arnoldi"
    assert picuda.ParameterScanPlan([1.0], build, task="spectrum").algorithm == "arnoldi"
    assert picuda.ParameterScanPlan([1.0], build, task="spectrum", algorithm="implicit_qr").algorithm == "iram"
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, task="spectrum", solver_options={"vectors": True})
    with pytest.raises(picuda.PiArgumentError):
        picuda.ParameterScanPlan([1.0], build, task="spectrum", algorithm="dense")


def test_arnoldi_continuation_vector():
    """scans.jl:1026-1041: v_1 + sum_{c >= 2} v_c / c over the selected modes, normalised;
    v_1 itself when the combination vanishes."""
    from picuda.scans import _arnoldi_continuation
    V = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], dtype=np.complex128)
    got = _arnoldi_continuation(V)
    ref = np.array([1, 1 / 2, 1 / 3, 0]) / np.linalg.norm([1, 1 / 2, 1 / 3])
    assert np.allclose(got, ref, atol=1e-15, rtol=0)
    W = np.array([[1, -2], [1, -2]], dtype=np.complex128)
    assert np.array_equal(_arnoldi_continuation(W), W[:, 0])
    assert np.array_equal(_arnoldi_continuation(V[:, :1]), V[:, 0])
