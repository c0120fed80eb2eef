"""Host logic of the DSL mirror: the ⋅ chain (written @), coefficient
collapse and the isotropy test that routes SymGrad⋅D⋅SymGrad to the
elastic kernel (src/multifield.jl:4814-4931)."""
import importlib

import numpy as np


def test_chain_and_isotropy(llf):
    dsl = importlib.import_module(llf.__name__ + ".dsl")
    llf.structured_box_mesh(n=1, order=1)
    p = llf.Problem([llf.Material("body")], type="Solid")
    t = llf.SymGrad(p) @ np.eye(6) @ 2.0 @ llf.SymGrad(p)
    assert isinstance(t, llf.BilinearTerm) and t.a.op == "SymGrad" and len(t.coef) == 2
    assert np.allclose(dsl._coefficient(t.coef), 2.0 * np.eye(6))
    assert isinstance(llf.Id(p) @ llf.Id(p), llf.BilinearTerm)
    lam, mu = 1.7, 0.9
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] = lam + 2 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    assert dsl._isotropic(D, 3) == (lam, mu)
    D[3, 4] = 0.1
    assert dsl._isotropic(D, 3) is None
    D2 = np.array([[lam + 2 * mu, lam, 0], [lam, lam + 2 * mu, 0], [0, 0, mu]])
    assert dsl._isotropic(D2, 2) == (lam, mu)
