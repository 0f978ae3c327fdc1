"""Galerkin symmetry Z = Z^T of the symmetric operators on one space (EFIE on RWG, Helmholtz single
layer and hypersingular on hats).

With the reference's far rules (3 test, 4 trial points) the matrix is symmetric only to the far
rules' error; with equal test and trial rules what remains is the Sauter-Schwab rules' error,
which falls with their order (about 4e-7 at the reference's n = 4, 3e-11 at n = 8).  The oracle
and both GPU precisions are held to that.
"""
import numpy as np
import pytest

import beastgpu_gb300 as bg
import oracle

SYM4 = bg.QuadStrat(far_test=4, far_trial=4, near_test=12, near_trial=12)
SYM8 = bg.QuadStrat(far_test=4, far_trial=4, near_test=12, near_trial=12, ss_cf=8, ss_ce=8, ss_cv=8)


def _cases():
    m = bg.icosphere(1)
    return [("efie", bg.Maxwell3D.singlelayer(wavenumber=2.0), bg.raviartthomas(m)),
            ("hh", bg.Helmholtz3D.singlelayer(wavenumber=2.0), bg.lagrangec0d1(m)),
            ("hs", bg.Helmholtz3D.hypersingular(wavenumber=2.0), bg.lagrangec0d1(m))]


def _asym(Z):
    return np.abs(Z - Z.T).max() / np.abs(Z).max()


@pytest.mark.parametrize("case", range(3))
def test_oracle_symmetry_follows_the_singular_rules(case):
    name, op, X = _cases()[case]
    a_ref = _asym(oracle.assemble(op, X, X, bg.QuadStrat()))
    a4 = _asym(oracle.assemble(op, X, X, SYM4))
    a8 = _asym(oracle.assemble(op, X, X, SYM8))
    assert a8 < 1e-10 < a4 < 1e-5 < a_ref, (name, a_ref, a4, a8)


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(3))
def test_gpu_symmetry(case):
    name, op, X = _cases()[case]
    Z = bg.assemble_gpu(op, X, X, quadstrat=SYM8)
    assert _asym(Z) < 1e-10, (name, _asym(Z))
    Zm = bg.assemble_gpu(op, X, X, bg.GPUConfiguration(precision="mixed"), quadstrat=SYM8)
    assert _asym(Zm) < 1e-6, (name, _asym(Zm))
