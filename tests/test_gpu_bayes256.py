"""The BAYESIAN workload at full size: 256x256x192, 20 rings, VROT and VDISP per ring with INC and PA global (42
dimensions), the ANALYTIC model (the reference's default for BAYESIAN), 1024 independent points in one device batch.

Parity: the sums of squares of a spread of members against the CPU oracle pipeline (its ANALYTIC model, FP64 direct
convolution and residual) within SS_RTOL, and every member of the 1024-point batch equal, bit for bit, to its value
in a batch of its own (independent points share nothing, so the batch size cannot change a result)."""
import numpy as np
import pytest

from test_gpu_likelihood import SS_RTOL, _oracle_ss

pytestmark = pytest.mark.gpu

NB = 1024
CHECKED = (0, 1, 337, 700, 1023)


@pytest.fixture(scope="module")
def bayes256():
    from bbarolo2_gb300 import bayesian, configs, engine
    cube, rings = configs.bayes256(galmodtype="ANALYTIC")
    dm = engine.DiskModel(cube, galmodtype="ANALYTIC")
    truth = dm.array(rings, seed=1)
    sigma = 0.01 * float(truth.max())
    g = np.random.default_rng(7)
    data = (truth + g.normal(0., sigma, truth.shape)).astype(np.float32)
    mask = truth > 3 * sigma
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    prob = bayesian.Problem(rings, per_ring=("vrot", "vdisp"), global_=("inc", "phi"),
                            priors={"vrot": (0., 350.), "vdisp": (1., 40.), "inc": (30., 80.), "phi": (0., 360.)})
    t0 = np.clip(prob.unit(np.r_[rings.vrot, rings.vdisp, rings.inc[0], rings.phi[0]])[0], 0, 1)
    u = np.clip(t0 + 0.01 * g.standard_normal((NB, prob.ndim)), 0., 1.)
    return dm, L, prob, rings, data, mask, u


def test_bayes256_batch_vs_oracle(gpu_lib, oracle_lib, bayes256):
    from oracle import oracle as O
    dm, L, prob, rings, data, mask, u = bayes256
    assert prob.ndim == 42
    rows = prob.rows(u)
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    ss, _ = L.run(sr, nv, descs, galmodtype="ANALYTIC")
    assert ss.shape == (NB,) and np.all(np.isfinite(ss)) and np.all(ss > 0)
    errs = []
    for k in CHECKED:
        ref = _oracle_ss(dm, O, sr[k], nv[k], boxes[k], 1, data, mask, 2, galmodtype="ANALYTIC")
        errs.append(abs(ss[k] - ref) / ref)
        assert abs(ss[k] - ref) <= SS_RTOL * ref, (k, ss[k], ref)
    print("bayes256: max relative error of the sum of squares", max(errs))
    # the members are distinct models: a batch that repeated one member would pass the spot checks above
    assert len(np.unique(ss)) == NB


def test_bayes256_members_independent_of_batch(gpu_lib, bayes256):
    dm, L, prob, rings, data, mask, u = bayes256
    rows = prob.rows(u)
    whole = L.evaluate(rows, rings, seed=1, galmodtype="ANALYTIC")
    for k in CHECKED:
        alone = L.evaluate(rows[k:k + 1], rings, seed=1, galmodtype="ANALYTIC")
        assert whole[k] == alone[0], (k, whole[k], alone[0])
    part = L.evaluate(rows[256:384], rings, seed=1, galmodtype="ANALYTIC")
    np.testing.assert_array_equal(whole[256:384], part)
