"""The fitting chain: synthesis -> rectification -> rotation -> LSF, differentiated through the
hand-written reverse modes and driven by L-BFGS-B (korg_gb300.fit, the pattern of
src/Fit/fit_via_synthesis.jl:304-390 for line strengths)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_fit_recovers_log_gf_through_rotation_and_lsf(gpu_lib):
    torch = pytest.importorskip("torch")
    pytest.importorskip("scipy")
    from korg_gb300 import synthetic
    from korg_gb300.fit import SpectrumModel, fit_log_gf
    w = synthetic.config0(seed=2, n_lines=300)
    w.wavelengths = (5000.0, 5020.0)
    w.linelist = synthetic.synthetic_linelist(300, 5001.0, 5019.0, seed=2)
    inp = synthetic.prepare(w)
    ctx = gpu_lib.Context(0)
    strong = np.argsort(-(inp.linelist.log_gf - 0.5 * inp.linelist.E_lower))[:3]
    obs_wls = np.arange(5002.0, 5018.0, 0.05)
    model = SpectrumModel(inp, strong, obs_wls=obs_wls, R=20000.0, vsini=5.0, precision="fp64", ctx=ctx)
    truth = model.initial() + np.array([0.15, -0.1, 0.05])
    obs = model(torch.as_tensor(truth, device=model.dev)).detach().cpu().numpy()
    fitted, loss, res = fit_log_gf(inp, obs, strong, obs_wls=obs_wls, R=20000.0, vsini=5.0, precision="fp64",
                                   ctx=ctx)
    np.testing.assert_allclose(fitted, truth, atol=1e-4)
    assert loss < 1e-10, (loss, res.message)
    ctx.close()
