"""Failure handling: bounded device loops reach Python as the documented warning or exception, bad
caller input stops on the host, and a failed emulator kernel sends its queries to the plain SAM.

Nothing here faults, traps or hangs a GPU: device-side limits are driven to exhaustion only through
their documented arguments (the gradient solve's sweep limit), and the other failures are made on the
host (fake status words, raising stand-ins)."""

import warnings

import numpy as np
import pytest

from conftest import load_golden


class _FakeStatus:
    def __init__(self, code):
        self.code = code
        self.resets = 0

    def read(self):
        return self.code

    def reset(self):
        self.code = 0
        self.resets += 1


@pytest.mark.parametrize("order, msg", [
    (np.arange(5), "indices"),                       # too short
    (np.array([0, 1, 2, 3, 4, 6]), "lie in"),         # out of range
    (np.array([0, 1, 2, 3, -1, 5]), "lie in"),        # negative
    (np.array([0, 1, 2, 3, 3, 5]), "exactly once"),   # a bin twice
    (np.linspace(0, 5, 6), "integer"),                # not indices
])
def test_caller_order_is_checked_on_the_host(order, msg):
    from holodeck_gb300 import cyutils
    with pytest.raises(ValueError, match=msg):
        cyutils.checked_order(order, 6)


def test_sampler_exhaustion_raises():
    from holodeck_gb300 import _native as N
    from holodeck_gb300 import cyutils
    cyutils._raise_status(_FakeStatus(0))
    cyutils._raise_status(_FakeStatus(N.STATUS_TABLE_RANGE))
    with pytest.raises(RuntimeError, match="attempt budget"):
        cyutils._raise_status(_FakeStatus(N.STATUS_ITERATION_LIMIT))


def test_realization_count_bound_is_checked_on_the_host(built_lib):
    """Realization counts beyond one launch's grid are rejected before anything is enqueued."""
    from holodeck_gb300 import _native as N
    lib = N.load()
    p = 16    # any non-null pointer: the call must return before touching it
    too_many = 65535 * 1024 + 1
    rc = lib.hgb_loudest_hc_from_sorted(p, p, 10, 2, too_many, 1, p, N.RNG_PHILOX, 0, None, p, p, p, 1 << 20, None,
                                        None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT
    rc = lib.hgb_sam_poisson_gwb(p, p, 10, 2, too_many, N.RNG_PHILOX, 0, None, p, p, 1 << 20, None, None)
    assert rc == N.HGB_ERR_INVALID_ARGUMENT


def test_mlp_status_raises_once_and_clears():
    from holodeck_gb300 import _native as N
    from holodeck_gb300.emulator import MLPEnsemble
    fake = type("Net", (), {})()
    fake.status = _FakeStatus(N.STATUS_ITERATION_LIMIT)
    with pytest.raises(N.NativeError, match="timed out"):
        MLPEnsemble.check_status(fake)
    assert fake.status.resets == 1
    MLPEnsemble.check_status(fake)                     # cleared: the next call passes
    with pytest.raises(N.NativeError):
        MLPEnsemble.check_status(fake, N.STATUS_ITERATION_LIMIT)   # a value read by the graphed path


def test_emulator_query_falls_back_when_the_network_fails():
    """A query whose network kernels timed out is re-solved by the fallback (every row); without a
    fallback the error reaches the caller."""
    from holodeck_gb300 import _native as N
    from holodeck_gb300.emulator import Emulator
    emu = Emulator.__new__(Emulator)
    emu.nfreqs = 3

    def failing_predict(params, spread_stats=None, **kwargs):
        raise N.NativeError("an MLP kernel timed out waiting for the tensor core")

    emu.predict = failing_predict
    params = np.zeros((4, 6))
    calls = []
    out, redo = emu.query(params, fallback=lambda row: calls.append(row) or np.full((3, 4), 7.0))
    assert redo.all() and len(calls) == 4 and np.all(out == 7.0)
    with pytest.raises(N.NativeError):
        emu.query(params)


@pytest.mark.gpu
def test_gradient_sweep_limit_warns(built_lib):
    """The scatter's gradient solve stopped after one sweep sets its status bit, which surfaces as
    scipy's non-convergence warning; the default limit converges silently."""
    from holodeck_gb300.sams import scatter as S
    g = load_golden("ref_scatter.npz")
    args = (g["s0_mtot"], g["s0_mrat"], g["s0_density_noscatter"], 0.28)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        S.add_scatter_to_masses(*args)
    with pytest.warns(UserWarning, match="did not converge"):
        S.add_scatter_to_masses(*args, maxiter=1)
    with pytest.raises(ValueError):
        S.add_scatter_to_masses(*args, maxiter=0)
