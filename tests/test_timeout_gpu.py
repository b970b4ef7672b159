"""The bounded-wait failure path of the tensor-core Legendre kernel, made
to run out on the host's request and without a GPU fault.

Every mbarrier wait of legendre_tc_kernel gives up after "wait_limit_ms";
the kernel then records an error code, stops issuing work, frees its TMEM
and returns, and the host reports DCCM_ERR_TIMEOUT.  The knob
"tc_withhold_loads" makes the kernel's load thread issue nothing, so the
MMA thread's first wait on a stage's "full" barrier (a phase nothing will
complete) runs out: no copy and no MMA is in flight when the CTAs leave.
The next call on the same plan, knobs reset, must be correct against the
oracle.  The reference's analogue is the fatal `stop` of
common/grid_mapping_util_jones99.f90:433-438; here nothing aborts.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TIMEOUT = -8


@pytest.mark.parametrize("prec", [1, 2])
def test_expired_wait_reports_timeout_then_recovers(dccm, oracle, synth, cuda, prec):
    torch = cuda
    N, I, J, B = 85, 256, 128, 16
    plan = dccm.ShtPlan(N, I, J, prec, max_batch=B)
    spec = synth.spectra(N, B, seed=5)
    go = oracle.sht_inverse(N, I, J, spec)
    ds = torch.from_numpy(spec.view(np.float64).copy()).cuda()
    dg = torch.empty((B, J, I), dtype=torch.float64, device="cuda")
    ds2 = torch.empty_like(ds)
    saved = {k: dccm.tune_get(k) for k in ("wait_limit_ms", "tc_withhold_loads")}
    try:
        dccm.tune_set("wait_limit_ms", 20)
        dccm.tune_set("tc_withhold_loads", 1)
        # device entry points: the launch succeeds, the status reports the expiry
        plan.inverse_dev(ds, dg, B)
        st, derr = plan.status()
        assert st == TIMEOUT and derr in (1, 2, 3, 4), (st, derr)
        assert plan.status() == (0, 0)  # reading the status cleared the flag
        plan.forward_dev(dg, ds2, B)
        st, derr = plan.status()
        assert st == TIMEOUT and derr != 0, (st, derr)
        # host entry point: the call itself returns the timeout
        with pytest.raises(dccm.DccmError) as e:
            plan.inverse(spec)
        assert e.value.status == TIMEOUT
        assert plan.status() == (0, 0)
    finally:
        for k, v in saved.items():
            dccm.tune_set(k, v)
    # the same plan afterwards: correct results, no error left behind
    plan.inverse_dev(ds, dg, B)
    plan.forward_dev(dg, ds2, B)
    torch.cuda.synchronize()
    assert plan.status() == (0, 0)
    assert rel_l2(dg.cpu().numpy(), go) <= 1e-6
    assert rel_l2(ds2.cpu().numpy().view(np.complex128), spec) <= 1e-6
    g = plan.inverse(spec)
    assert rel_l2(g, go) <= 1e-6

