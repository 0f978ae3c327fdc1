"""Boundary integral operators and quadrature strategies, BEAST-style.

Mirrors the constructors a BEAST user calls (`Helmholtz3D.singlelayer(wavenumber=k)`,
`Helmholtz3D.doublelayer`, `.doublelayer_transposed`, `.hypersingular`,
`Maxwell3D.singlelayer(wavenumber=k)`, `Maxwell3D.doublelayer(wavenumber=k)`) and the
operator fields the reference reads (`biop.alpha`, `biop.gamma`,
doubleQuadRuleMainCase.jl:168-169; SauterSchwab.jl:319-320).  The Green function is
G(R) = exp(-gamma R) / (4 pi R) with gamma = i k.
"""
from __future__ import annotations

from dataclasses import dataclass

OP_HELMHOLTZ3D_SL = 0
OP_MAXWELL3D_SL = 1
OP_MAXWELL3D_DL = 2
OP_HELMHOLTZ3D_DL = 3
OP_HELMHOLTZ3D_DLT = 4
OP_HELMHOLTZ3D_HS = 5

_NAMES = {OP_HELMHOLTZ3D_SL: "Helmholtz3D.singlelayer", OP_MAXWELL3D_SL: "Maxwell3D.singlelayer",
          OP_MAXWELL3D_DL: "Maxwell3D.doublelayer", OP_HELMHOLTZ3D_DL: "Helmholtz3D.doublelayer",
          OP_HELMHOLTZ3D_DLT: "Helmholtz3D.doublelayer_transposed",
          OP_HELMHOLTZ3D_HS: "Helmholtz3D.hypersingular"}


@dataclass(frozen=True)
class Operator:
    kind: int
    alpha: complex
    gamma: complex
    beta: complex = 0.0

    @property
    def wavenumber(self) -> float:
        return (self.gamma / 1j).real

    def __repr__(self):
        return f"{_NAMES[self.kind]}(alpha={self.alpha}, beta={self.beta}, gamma={self.gamma})"


def _gamma(gamma, wavenumber):
    if gamma is None and wavenumber is None:
        raise ValueError("give gamma or wavenumber")
    if gamma is None:
        gamma = 1j * wavenumber
    return complex(gamma)


class Helmholtz3D:
    @staticmethod
    def singlelayer(*, wavenumber=None, gamma=None, alpha=None) -> Operator:
        """alpha * int int G(x, y) f(x) g(y); alpha defaults to 1 (BEAST)."""
        g = _gamma(gamma, wavenumber)
        return Operator(OP_HELMHOLTZ3D_SL, complex(1.0 if alpha is None else alpha), g)

    @staticmethod
    def doublelayer(*, wavenumber=None, gamma=None, alpha=None) -> Operator:
        """K: alpha * int int f(x) dG/dn_y(x, y) g(y), dG/dn_y = n_y . grad_y G; alpha defaults to 1."""
        return Operator(OP_HELMHOLTZ3D_DL, complex(1.0 if alpha is None else alpha), _gamma(gamma, wavenumber))

    @staticmethod
    def doublelayer_transposed(*, wavenumber=None, gamma=None, alpha=None) -> Operator:
        """K': alpha * int int f(x) dG/dn_x(x, y) g(y), dG/dn_x = n_x . grad_x G; alpha defaults to 1."""
        return Operator(OP_HELMHOLTZ3D_DLT, complex(1.0 if alpha is None else alpha), _gamma(gamma, wavenumber))

    @staticmethod
    def hypersingular(*, wavenumber=None, gamma=None, alpha=None, beta=None) -> Operator:
        """W in Maue's form: int int G [alpha (n_x . n_y) f g + beta curl f . curl g];
        alpha defaults to gamma^2 and beta to 1."""
        g = _gamma(gamma, wavenumber)
        return Operator(OP_HELMHOLTZ3D_HS, g * g if alpha is None else complex(alpha), g,
                        1.0 if beta is None else complex(beta))


class Maxwell3D:
    @staticmethod
    def singlelayer(*, wavenumber=None, gamma=None, alpha=None, beta=None) -> Operator:
        """EFIE operator: int int G [alpha f.g + beta div f div g]; alpha = -gamma, beta = -1/gamma."""
        g = _gamma(gamma, wavenumber)
        a = -g if alpha is None else complex(alpha)
        b = -1.0 / g if beta is None else complex(beta)
        return Operator(OP_MAXWELL3D_SL, a, g, b)

    @staticmethod
    def doublelayer(*, wavenumber=None, gamma=None, alpha=None) -> Operator:
        """MFIE operator K: alpha int int f(x) . (grad_x G(x, y) x g(y)); alpha defaults to 1."""
        g = _gamma(gamma, wavenumber)
        return Operator(OP_MAXWELL3D_DL, complex(1.0 if alpha is None else alpha), g)


@dataclass(frozen=True)
class QuadStrat:
    """Quadrature strategy, the fields of BEAST's DoubleNumWiltonSauterQStrat as used here.

    far_test / far_trial: points of the symmetric triangle rules for far pairs (the
    reference hard-codes 3 and 4, GPU_scheduler.jl:94-95); near_test / near_trial: rules for
    near pairs; ss_cf / ss_ce / ss_cv: Gauss-Legendre points per dimension of the 4-D
    Sauter-Schwab rules (the reference hard-codes 4, SauterSchwab.jl:331,433).
    Supported triangle rules: 1, 3, 4, 6, 7, 12, 13 points.
    """
    far_test: int = 3
    far_trial: int = 4
    near_test: int = 12
    near_trial: int = 13
    ss_cf: int = 4
    ss_ce: int = 4
    ss_cv: int = 4


def defaultquadstrat(op=None, test=None, trial=None) -> QuadStrat:
    return QuadStrat()
