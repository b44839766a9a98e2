"""FP64 mode (the reference run errors are measured against) versus the
oracle's FP64 restatement of the same algorithm."""
import numpy as np
import pytest

import trace_gb300 as tg
from oracle import oracle as O
from tests._util import rel_l2, theta_uniform

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("alg,kw", [("sirt", {}), ("mlem", {}), ("pml", {"beta": 0.3}),
                                    ("apmlr", {"beta": 0.3, "beta1": 0.5})])
def test_fp64_mode_matches_fp64_oracle(alg, kw):
    C, P, S, n = 48, 40, 3, 4
    th = theta_uniform(P)
    tabs = O.angle_table(th)
    rng = np.random.default_rng(4)
    sino = rng.uniform(0.5, 2.0, (P, S, C)).astype(np.float32)
    want = O.run(alg, sino, tables=tabs, n_iter=n, precision=O.F64, **kw)["recon"]
    plan = tg.Plan(P, S, C, th, mode="fp64")
    plan.set_sinogram(sino, apply_abs=alg != "sirt")
    plan.reset_recon(alg)
    plan.iterate(alg, n, tg.default_params(alg, **kw))
    got = plan.get_recon(alg)
    assert rel_l2(got, want) < 1e-6
    f32 = O.run(alg, sino, tables=tabs, n_iter=n, **kw)["recon"]
    assert rel_l2(f32, want) > 0  # the float run is a different computation
    plan.close()


def test_fp64_mode_rejects_operator_calls_and_16bit():
    th = theta_uniform(12)
    with pytest.raises(tg.TraceError):
        tg.Plan(12, 1, 16, th, mode="fp64", len_storage="u16")
    plan = tg.Plan(12, 1, 16, th, mode="fp64")
    plan.reset_recon("sirt")
    with pytest.raises(tg.TraceError) as e:
        plan.reduce("sirt")
    assert e.value.status == 4
    plan.close()
