"""Element-category objective terms on the host side of the GPU path.

The GPU returns each element's centroid strain, stress and volume
(``asend_element_fields``); this module applies the reference's operator to
them and turns dL/dq into the per-element weights dL/dsigma, dL/deps that the
adjoint takes (``asend_set_element_objective``).

Reference: ObjectiveTerm (objective_meth.rs)
  * q per element: 'stress' / 'strain' component, or 'strainEnergy'
    = 1/2 sigma . eps (get_obj_val :665-720);
  * operators: powerNorm coef (sum (q - t)^p)^(1/p) (:329-337), ks
    coef/p ln sum exp(p q / t) (:390-398, q divided by its target at :645-648),
    volumeIntegral coef (sum q V - t_0)^p (:442-449), volumeAverage
    coef (sum q V / sum V - t_0)^p (:504-516);
  * targets (get_tgt_vec :94-215): one value for all, one per element, or
    none (0; 1 for ks);
  * derivatives: getd_ld_u :1051-1160 and the d_*d_u helpers :339-503 give
    dL/dq_e g_e; the strain-energy weights 1/2 eps, 1/2 sigma follow
    :1087-1104.
"""
from __future__ import annotations

import numpy as np

CATEGORIES = ("stress", "strain", "strainEnergy")
OPERATORS = ("powerNorm", "ks", "volumeIntegral", "volumeAverage")


def element_values(eps, sig, category, component=0):
    """q per element [n] from centroid strains and stresses [n, 6]."""
    if category == "stress":
        return sig[:, component - 1]
    if category == "strain":
        return eps[:, component - 1]
    if category == "strainEnergy":
        return 0.5 * np.einsum("ij,ij->i", sig, eps)
    raise NotImplementedError(f"objective category {category} is not on the GPU path")


def targets_for(n, operator, targets):
    t = np.asarray(targets if targets is not None else [], dtype=np.float64).ravel()
    if len(t) == n:
        return t.copy()
    if len(t) == 1:
        return np.full(n, t[0])
    if len(t) == 0:
        return np.full(n, 1.0 if operator == "ks" else 0.0)
    raise ValueError(f"{len(t)} targets for {n} elements")


def operator_value(q, vol, tgt, operator, coef, exponent):
    """(L, g = dL/dq per element)."""
    p = float(exponent)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        if operator == "powerNorm":
            ps = np.sum(np.power(q - tgt, p))
            L = coef * ps ** (1.0 / p)
            g = coef * ps ** (1.0 / p - 1.0) * np.power(q - tgt, p - 1.0)
        elif operator == "ks":
            ex = np.exp(p * q / tgt)
            s = ex.sum()
            L = (coef / p) * np.log(s)
            g = coef * ex / s / tgt
        elif operator == "volumeIntegral":
            base = np.sum(q * vol) - tgt[0]
            L = coef * base ** p
            g = coef * p * base ** (p - 1.0) * vol
        elif operator == "volumeAverage":
            tv = vol.sum()
            base = np.sum(q * vol) / tv - tgt[0]
            L = coef * base ** p
            g = coef * p * base ** (p - 1.0) * vol / tv
        else:
            raise NotImplementedError(f"objective operator {operator} is not on the GPU path")
    return float(L), g


def element_term(eps, sig, vol, elems, category, component=0, operator="powerNorm", coef=1.0, exponent=1.0,
                 targets=None):
    """Value and adjoint weights of one term over the elements ``elems``.

    eps, sig: [n_el, 6] centroid fields; vol: [n_el].  Returns (L, w_stress,
    w_strain) with the weights [n_el, 6] (zero outside the set)."""
    elems = np.asarray(elems, dtype=np.int64)
    n_el = eps.shape[0]
    if category not in CATEGORIES:
        raise NotImplementedError(f"objective category {category} is not on the GPU path")
    if category != "strainEnergy" and not 1 <= component <= 6:
        raise ValueError(f"{category} objective needs a component 1-6")
    e, s, v = eps[elems], sig[elems], vol[elems]
    q = element_values(e, s, category, component)
    tgt = targets_for(len(elems), operator, targets)
    L, g = operator_value(q, v, tgt, operator, coef, exponent)
    wa = np.zeros((n_el, 6))
    wb = np.zeros((n_el, 6))
    if category == "stress":
        np.add.at(wa[:, component - 1], elems, g)
    elif category == "strain":
        np.add.at(wb[:, component - 1], elems, g)
    else:
        np.add.at(wa, elems, 0.5 * g[:, None] * e)
        np.add.at(wb, elems, 0.5 * g[:, None] * s)
    return L, wa, wb
