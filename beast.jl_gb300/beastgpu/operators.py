"""Operators, excitations and quadrature strategies: host mirror of BEAST's API.

  Maxwell3D.singlelayer / doublelayer / planewave   src/maxwell/maxwell.jl:16-95
  Helmholtz3D.singlelayer / doublelayer / doublelayer_transposed / planewave
                                                      src/helmholtz3d/helmholtz3d.jl:7-119
  n x K  (DoubleLayerRotatedMW3D)                    src/maxwell/nxdbllayer.jl:17-44
  Identity / NCross local operators                  src/identityop.jl:7-24
  DoubleNumWiltonSauterQStrat / DoubleNumSauterQstrat / DoubleNumQStrat
                                                      src/quadrature/*.jl
  gamma / wavenumber handling                        src/maxwell/mwops.jl:213-273
"""
from dataclasses import dataclass

from . import spaces as _sp

# operator kind codes shared with the C ABI (include/beastgpu.h)
MW_SL, MW_DL, MW_NXDL, HH_SL, HH_DL, HH_DLT = 1, 2, 3, 4, 5, 6
QS_WILTON_SAUTER, QS_SAUTER, QS_DOUBLENUM = 1, 2, 3
QS_TEST_REFINES_TRIAL, QS_TRIAL_REFINES_TEST = 4, 5


def gamma_wavenumber_handler(gamma, wavenumber):
    """src/maxwell/mwops.jl:213-244"""
    if gamma is not None and wavenumber is not None:
        raise ValueError("Supplying both gamma and wavenumber is not supported.")
    if gamma is None and wavenumber is None:
        return 0.0, 0.0  # static problem (Val(0))
    if gamma is None:
        wavenumber = complex(wavenumber)
        if wavenumber.real == 0:
            gamma = -wavenumber.imag
        else:
            gamma = 1j * wavenumber
    else:
        gamma = complex(gamma)
        wavenumber = gamma.imag if gamma.real == 0 else -1j * gamma
    return complex(gamma), wavenumber


@dataclass(frozen=True)
class IntegralOperator:
    kind: int
    gamma: complex
    alpha: complex = 1.0
    beta: complex = 0.0

    def __rmul__(self, s):
        return LinearCombination([(complex(s), self)])

    def __add__(self, other):
        return LinearCombination([(1.0, self)]) + other

    def __sub__(self, other):
        return LinearCombination([(1.0, self)]) + (-1.0) * other

    def __neg__(self):
        return (-1.0) * self


@dataclass(frozen=True)
class LocalOperator:
    which: int  # 0 Identity, 1 NCross

    def __rmul__(self, s):
        return LinearCombination([(complex(s), self)])

    def __neg__(self):
        return (-1.0) * self


class LinearCombination:
    """src/operator.jl:27-75 (sum of scaled operators; assembled term by term into one store)"""

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        if isinstance(other, LinearCombination):
            return LinearCombination(self.terms + other.terms)
        return LinearCombination(self.terms + [(1.0, other)])

    def __sub__(self, other):
        return self + (-1.0) * other

    def __rmul__(self, s):
        return LinearCombination([(complex(s) * c, op) for (c, op) in self.terms])


def Identity():
    return LocalOperator(0)


def NCross():
    return LocalOperator(1)


class Maxwell3D:
    @staticmethod
    def singlelayer(gamma=None, wavenumber=None, alpha=None, beta=None):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        if g == 0:
            assert alpha is not None and beta is not None
        alpha = -g if alpha is None else alpha
        beta = -1.0 / g if beta is None else beta
        return IntegralOperator(MW_SL, complex(g), complex(alpha), complex(beta))

    @staticmethod
    def doublelayer(gamma=None, wavenumber=None, alpha=None):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        return IntegralOperator(MW_DL, complex(g), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def planewave(direction, polarization, wavenumber, amplitude=1.0):
        return PlaneWaveMW(tuple(direction), tuple(polarization), 1j * wavenumber,
                           complex(amplitude))


def nxdoublelayer(gamma=None, wavenumber=None, alpha=1.0):
    """n x K = DoubleLayerRotatedMW3D(alpha, gamma)"""
    g, _ = gamma_wavenumber_handler(gamma, wavenumber)
    return IntegralOperator(MW_NXDL, complex(g), complex(alpha))


class Helmholtz3D:
    @staticmethod
    def singlelayer(gamma=None, wavenumber=None, alpha=None):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        return IntegralOperator(HH_SL, complex(g), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def doublelayer(gamma=None, wavenumber=None, alpha=None):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        return IntegralOperator(HH_DL, complex(g), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def doublelayer_transposed(gamma=None, wavenumber=None, alpha=None):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        return IntegralOperator(HH_DLT, complex(g), complex(1.0 if alpha is None else alpha))

    @staticmethod
    def planewave(direction, gamma=None, wavenumber=None, amplitude=1.0):
        g, _ = gamma_wavenumber_handler(gamma, wavenumber)
        return PlaneWaveHH(tuple(direction), complex(g), complex(amplitude))


@dataclass(frozen=True)
class PlaneWaveMW:
    """src/maxwell/mwexc.jl:1-52: E(x) = a exp(-gamma d.x) u"""
    direction: tuple
    polarization: tuple
    gamma: complex
    amplitude: complex = 1.0


@dataclass(frozen=True)
class PlaneWaveHH:
    direction: tuple
    gamma: complex
    amplitude: complex = 1.0


# excitation kinds of the C ABI
EXC_TANGTRACE_E, EXC_CROSSTRACE_H, EXC_HH_DIRICHLET = 0, 1, 2


@dataclass(frozen=True)
class Excitation:
    """tested field: (n x E) x n  (TangTraceMW), n x H (CrossTraceMW of H = -1/(ik) curl E)
    or the Helmholtz Dirichlet trace of a plane wave"""
    kind: int
    wave: object


def tangential_trace(E):
    return Excitation(EXC_TANGTRACE_E, E)


def cross_trace_H(E):
    return Excitation(EXC_CROSSTRACE_H, E)


def dirichlet_trace(f):
    return Excitation(EXC_HH_DIRICHLET, f)


@dataclass(frozen=True)
class DoubleNumWiltonSauterQStrat:
    outer_rule_far: int
    inner_rule_far: int
    outer_rule_near: int
    inner_rule_near: int
    sauter_schwab_common_tetr: int
    sauter_schwab_common_face: int
    sauter_schwab_common_edge: int
    sauter_schwab_common_vert: int

    def orders(self):
        return (QS_WILTON_SAUTER, self.outer_rule_far, self.inner_rule_far, self.outer_rule_near,
                self.inner_rule_near, self.sauter_schwab_common_tetr,
                self.sauter_schwab_common_face, self.sauter_schwab_common_edge,
                self.sauter_schwab_common_vert)


@dataclass(frozen=True)
class DoubleNumSauterQstrat:
    outer_rule: int
    inner_rule: int
    sauter_schwab_common_tetr: int
    sauter_schwab_common_face: int
    sauter_schwab_common_edge: int
    sauter_schwab_common_vert: int

    def orders(self):
        return (QS_SAUTER, self.outer_rule, self.inner_rule, self.outer_rule, self.inner_rule,
                self.sauter_schwab_common_tetr, self.sauter_schwab_common_face,
                self.sauter_schwab_common_edge, self.sauter_schwab_common_vert)


@dataclass(frozen=True)
class DoubleNumQStrat:
    outer_rule: int
    inner_rule: int

    def orders(self):
        return (QS_DOUBLENUM, self.outer_rule, self.inner_rule, self.outer_rule,
                self.inner_rule, 0, 0, 0, 0)


@dataclass(frozen=True)
class TestRefinesTrialQStrat:
    """src/quadrature/strategies/testrefinestrialqstrat.jl:1-17: the test space lives on a
    refinement of the trial space's mesh; pairs that share a vertex integrate the trial cell's
    children with the wrapped strategy (rules/testrefinestrialqrule.jl:6-52)"""
    __test__ = False  # not a pytest class
    conforming_qstrat: DoubleNumWiltonSauterQStrat

    def orders(self):
        if not isinstance(self.conforming_qstrat, DoubleNumWiltonSauterQStrat):
            raise ValueError("TestRefinesTrialQStrat wraps a DoubleNumWiltonSauterQStrat")
        return (QS_TEST_REFINES_TRIAL,) + self.conforming_qstrat.orders()[1:]


@dataclass(frozen=True)
class TrialRefinesTestQStrat:
    """src/quadrature/strategies/trialrefinestestqstrat.jl:1-17: the same with the trial space
    on the refinement (rules/trialrefinestestqrule.jl:6-40)"""
    conforming_qstrat: DoubleNumWiltonSauterQStrat

    def orders(self):
        if not isinstance(self.conforming_qstrat, DoubleNumWiltonSauterQStrat):
            raise ValueError("TrialRefinesTestQStrat wraps a DoubleNumWiltonSauterQStrat")
        return (QS_TRIAL_REFINES_TEST,) + self.conforming_qstrat.orders()[1:]


def defaultquadstrat(op, tspace, bspace):
    """src/maxwell/mwops.jl:55, src/maxwell/nxdbllayer.jl:23, src/helmholtz3d/hh3dops.jl:92-93,
    src/integralop.jl:3-4"""
    if op.kind == MW_NXDL:
        return DoubleNumQStrat(6, 7)
    if op.kind in (MW_SL, MW_DL) and tspace.kind == _sp.RT and bspace.kind == _sp.RT:
        return DoubleNumWiltonSauterQStrat(2, 3, 6, 7, 5, 5, 4, 3)
    if op.kind in (HH_SL, HH_DL, HH_DLT) and tspace.kind in (_sp.P0, _sp.P1) \
            and bspace.kind in (_sp.P0, _sp.P1):
        return DoubleNumWiltonSauterQStrat(2, 3, 2, 3, 4, 4, 4, 4)
    return DoubleNumSauterQstrat(2, 3, 5, 5, 4, 3)
