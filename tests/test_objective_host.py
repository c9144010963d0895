"""Host side of the element-category objective terms
(asend3d_gb300/objective.py): the per-element weights dL/dsigma, dL/deps
against central differences of the operator value, treating the centroid
stresses and strains as independent inputs (1e-7 relative), plus the
target rules of get_tgt_vec (objective_meth.rs:94-215)."""
import numpy as np
import pytest

from asend3d_gb300.objective import element_term, targets_for

CASES = [("strainEnergy", 0, "volumeIntegral", 2.0, 1.0, None),
         ("strainEnergy", 0, "powerNorm", 1.0, 2.0, None),
         ("stress", 2, "powerNorm", 1.0, 3.0, [0.1]),
         ("strain", 5, "ks", 1.0, 4.0, [2.0]),
         ("stress", 4, "volumeAverage", 3.0, 2.0, [0.5]),
         ("strainEnergy", 0, "ks", 0.5, 8.0, None)]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[2]}" for c in CASES])
def test_weights_match_differences(case):
    cat, comp, op, coef, ex, tg = case
    rng = np.random.default_rng(5)
    n = 12
    eps = rng.standard_normal((n, 6))
    sig = rng.standard_normal((n, 6))
    vol = rng.uniform(0.5, 1.5, n)
    els = np.arange(1, n, 2) if op in ("powerNorm", "ks") else np.arange(n)
    if op == "powerNorm" and ex != 2.0:
        sig = np.abs(sig) + 0.5  # real powers of positive errors
    L, wa, wb = element_term(eps, sig, vol, els, cat, comp, op, coef, ex, tg)
    assert np.all(wa[np.setdiff1d(np.arange(n), els)] == 0)
    de = rng.standard_normal((n, 6))
    ds = rng.standard_normal((n, 6))
    h = 1e-6
    lp = element_term(eps + h * de, sig + h * ds, vol, els, cat, comp, op, coef, ex, tg)[0]
    lm = element_term(eps - h * de, sig - h * ds, vol, els, cat, comp, op, coef, ex, tg)[0]
    fd = (lp - lm) / (2 * h)
    assert np.sum(wa * ds) + np.sum(wb * de) == pytest.approx(fd, rel=1e-7, abs=1e-10 * abs(L))


def test_target_rules():
    assert np.all(targets_for(3, "powerNorm", None) == 0.0)
    assert np.all(targets_for(3, "ks", []) == 1.0)
    assert np.all(targets_for(3, "ks", [2.0]) == 2.0)
    assert np.all(targets_for(3, "powerNorm", [1, 2, 3]) == [1, 2, 3])
    with pytest.raises(ValueError):
        targets_for(3, "powerNorm", [1, 2])


def test_unsupported_categories():
    e = np.zeros((2, 6))
    with pytest.raises(NotImplementedError):
        element_term(e, e, np.ones(2), [0], "mises")
    with pytest.raises(NotImplementedError):
        element_term(e, e, np.ones(2), [0], "strainEnergy", operator="max")
    with pytest.raises(ValueError):
        element_term(e, e, np.ones(2), [0], "stress", 0)
