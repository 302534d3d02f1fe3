"""The bounded-wait failure path of the streamed operator kernel, made to run on purpose.

With the consumers' stage-wait limit cut to 2 microseconds and the producer holding back its
second stage for 200 microseconds, the consumers give up: the kernel sets its device error
bit, the producer stops issuing stages, waits for the copies it already issued and returns, and
fvm_rhs reports FVM_ERR_CUDA at its synchronisation.  No wait is unbounded and nothing faults:
the next normal call on the same problem runs and matches the oracle."""
import numpy as np
import pytest

import fvm_oracle as O
from problems import api_problem, oracle_problem, parity_error, rhs_term_scale, sine_diffusion

pytestmark = pytest.mark.gpu


def test_stream_wait_runs_out_reports_and_recovers(gpu_lib):
    import fvmgpu as F

    lib = gpu_lib.load()
    spec = sine_diffusion(400)  # 160k vertices: several stages per CTA
    prob = api_problem(spec)
    u = spec.u0 + 0.05 * np.sin(3 * spec.tri.points[:, 0])
    ref = O.fvm_eqs(oracle_problem(spec), u, 0.0)
    scale = rhs_term_scale(oracle_problem(spec), u, 0.0)
    F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0)  # warm (first-use set-up outside the test window)
    assert lib.fvm_test_set_stream_waits(2_000, 200_000) == 0
    try:
        with pytest.raises(gpu_lib.FVMError) as e:
            F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0)
        assert e.value.code == gpu_lib.FVM_ERR_CUDA
        assert "timed out" in str(e.value)
    finally:
        assert lib.fvm_test_set_stream_waits(0, 0) == 0
    for _ in range(2):
        du = F.fvm_eqs(np.zeros_like(u), u.copy(), prob, 0.0)
        assert parity_error(du, ref, scale) <= 1e-12


def test_stream_wait_settings_are_bounded(gpu_lib):
    lib = gpu_lib.load()
    assert lib.fvm_test_set_stream_waits(50, 0) == gpu_lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_test_set_stream_waits(0, 20_000_000) == gpu_lib.FVM_ERR_INVALID_ARGUMENT
    assert lib.fvm_test_set_stream_waits(0, 0) == 0
