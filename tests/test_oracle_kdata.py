"""The oracle's K data (build_K_data, run_gap_transport_scan.jl:297-305) pinned by the
reference's own tests of its parts:

* const_integral_term_A against direct quadrature of p^2/E on [0, Lambda]
  (tests/unit/relaxtime/test_oneloopintegrals.jl:125-131);
* A against adaptive quadrature of its integrand and against twice the nodes
  (test_oneloopintegrals.jl:133-159, with its TEST_PARAMS and 128 nodes on [0, 20]);
* calculate_G_from_A's formula and calculate_effective_couplings' limits -- K = 0 and
  G^f = 0 give K_alpha = G, G^u = G^s makes the pi, K and eta_8 channels degenerate with no
  0-8 mixing -- and the sign of det K at the reference's standard point
  (tests/unit/relaxtime/test_effective_couplings.jl:36-160, 160-200).
"""
import numpy as np
import pytest
from scipy.integrate import quad

from oracle import oracle as orc

HBARC = 197.327
TEST_PARAMS = dict(m1=0.24, mu1=0.12, T=0.17, Phi=0.15, Phibar=0.15)


@pytest.fixture(scope="module")
def P():
    return orc.default_params()


def test_const_integral_term_matches_quadrature(P):
    for m in (TEST_PARAMS["m1"], 0.38, 1.7, 1e-15):
        num, _ = quad(lambda p: p * p / np.sqrt(p * p + m * m), 0.0, P.Lambda, epsabs=1e-13, epsrel=1e-12)
        assert orc.const_integral_term_A(P, m) == pytest.approx(num, rel=1e-9, abs=1e-11)


def test_one_loop_A_matches_quadrature(P):
    m, mu, T, Phi, Phib = (TEST_PARAMS[k] for k in ("m1", "mu1", "T", "Phi", "Phibar"))
    p, w = orc.gauleg(0.0, 20.0, 128)
    result = orc.one_loop_A(P, p, w, m, mu, T, Phi, Phib)

    def integrand(q):
        E = np.sqrt(q * q + m * m)
        y = np.exp(-(E - mu) / T)
        z = np.exp(-(E + mu) / T)
        fp = (Phi * y + 2 * Phib * y * y + y ** 3) / (1 + 3 * Phi * y + 3 * Phib * y * y + y ** 3)
        fm = (Phib * z + 2 * Phi * z * z + z ** 3) / (1 + 3 * Phib * z + 3 * Phi * z * z + z ** 3)
        return q * q / E * (fp + fm)

    dist, _ = quad(integrand, 0.0, 20.0, epsabs=1e-10, epsrel=1e-8, limit=200)
    expected = 4.0 * (-orc.const_integral_term_A(P, m) + dist)
    assert result == pytest.approx(expected, rel=5e-5, abs=1e-6)
    p2, w2 = orc.gauleg(0.0, 20.0, 256)
    assert result == pytest.approx(orc.one_loop_A(P, p2, w2, m, mu, T, Phi, Phib), rel=5e-5, abs=1e-6)


def test_effective_couplings_limits(P):
    G, K = P.G, P.K
    for k0 in (orc.effective_couplings(G, 0.0, -0.3, -0.2), orc.effective_couplings(G, K, 0.0, 0.0)):
        for name in ("K0_plus", "K0_minus", "K123_plus", "K123_minus", "K4567_plus", "K4567_minus", "K8_plus",
                     "K8_minus"):
            assert abs(k0[name] - G) < 1e-15, name
        assert abs(k0["K08_plus"]) < 1e-15 and abs(k0["K08_minus"]) < 1e-15
    sym = orc.effective_couplings(G, K, -0.25, -0.25)
    assert abs(sym["K123_plus"] - sym["K4567_plus"]) < 1e-15
    assert abs(sym["K123_minus"] - sym["K4567_minus"]) < 1e-15
    assert abs(sym["K123_plus"] - sym["K8_plus"]) < 1e-15
    assert abs(sym["K123_minus"] - sym["K8_minus"]) < 1e-15
    assert abs(sym["K08_plus"]) < 1e-15 and abs(sym["K08_minus"]) < 1e-15
    # magnitudes at G^u = -0.3, G^s = -0.2 (test_effective_couplings.jl:84-100)
    kc = orc.effective_couplings(G, K, -0.3, -0.2)
    for name, v in kc.items():
        if name.startswith("det"):
            assert np.isfinite(v) and v > 0
        elif name.startswith("K08"):
            assert abs(v) < 0.1 * G
        else:
            assert abs(v - G) / G < 0.5
    assert kc["det_K_plus"] == pytest.approx(kc["K0_plus"] * kc["K8_plus"] - kc["K08_plus"] ** 2, rel=1e-15)


def test_kdata_at_the_standard_point(P):
    """T = 150 MeV, mu = 0, m_u = 300 MeV, m_s = 500 MeV, Phi = Phibar = 0.5 (the reference's
    standard test point): G^f = -N_c/(4 pi^2) m_f A_f and det K > 0 in both channels; the
    temperature scan of the same test keeps det K^- > 0 and the couplings finite."""
    for T_MeV in (50.0, 100.0, 150.0, 200.0, 250.0):
        masses = np.array([[300.0, 300.0, 500.0]]) / HBARC
        kd = orc.kdata(P, [T_MeV / HBARC], [0.0], [0.0], masses, [[0, 0, 0, 0.5, 0.5]])
        for v in kd.values():
            assert np.isfinite(v[0])
        assert kd["det_K_minus"][0] > 0
        if T_MeV == 150.0:
            assert kd["det_K_plus"][0] > 0
        assert kd["A_d"][0] == kd["A_u"][0]
        assert kd["G_u"][0] == pytest.approx(-3.0 / (4 * np.pi ** 2) * masses[0, 0] * kd["A_u"][0], rel=1e-15)
        assert kd["G_s"][0] == pytest.approx(-3.0 / (4 * np.pi ** 2) * masses[0, 2] * kd["A_s"][0], rel=1e-15)
