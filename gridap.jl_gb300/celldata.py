"""Weak forms as small expression trees, recognised into the closed set of integrands the
device kernels evaluate.

Gridap builds cell arrays lazily from Julia expressions such as
`∫( κ*∇(v)⋅∇(u) )dΩ` (CellData/CellQuadratures.jl:138-202). The drop-in cannot ship
arbitrary Julia code to the GPU, so it recognises the integrands it provides and passes an
enum plus coefficient arrays across the C ABI:

  - bilinear  `κ * inner(grad(v), grad(u))`  (κ: number, per-cell CellField, or absent);
  - linear    `f * v`  (f: number, NodalField, SinSum, or a Python callable of x);
  - bilinear  `inner(ε(v), σ(ε(u)))` with σ = isotropic_stress(λ, μ), i.e.
              ε(v) ⊙ (λ tr(ε(u)) I + 2μ ε(u))  (λ, μ: numbers or per-cell CellFields);
  - linear    `inner(f, v)` with f a constant 3-vector (body force);
  - on a BoundaryTriangulation measure: sums of  c v u,  c v (n⋅∇u),  c (n⋅∇v) u,
    c (n⋅∇v)(n⋅∇u)  (c constant; Nitsche and Robin terms) in bilinear forms and of
    g v,  g (n⋅∇v)  in linear forms (g a number, a callable of x, or n⋅G with G a callable
    returning vectors, e.g. the gradient of an exact solution).

Anything else raises NotImplementedError; in Gridap that integrand would stay on Gridap's
own CPU path.
"""
from __future__ import annotations

import numpy as np


class CellField:
    """A field with one value per cell (piecewise constant), e.g. a per-cell coefficient."""

    def __init__(self, values, trian=None):
        self.values = values
        self.trian = trian


class NodalField:
    """A Q1 FE function given by its values at every mesh node (node order)."""

    def __init__(self, values, model=None):
        self.values = values
        self.model = model


class SinSum:
    """f(x) = sum_k a_k prod_d sin(pi m_kd x_d); `terms` rows are (a_k, m_k1, ..., m_kD)."""

    def __init__(self, terms):
        self.terms = np.asarray(terms, dtype=np.float64)

    def __call__(self, x):
        x = np.atleast_2d(x)
        D = x.shape[1]
        out = np.zeros(x.shape[0])
        for t in self.terms:
            p = np.full(x.shape[0], t[0])
            for d in range(D):
                p = p * np.sin(np.pi * t[1 + d] * x[:, d])
            out += p
        return out


class _Expr:
    def __mul__(self, other):
        if isinstance(other, _Expr):
            return _Prod(self, other)
        return _Scaled(other, self)

    def __rmul__(self, other):
        return _Scaled(other, self)

    def __add__(self, other):
        return _Sum([(1.0, self), (1.0, other)])

    def __sub__(self, other):
        return _Sum([(1.0, self), (-1.0, other)])

    def __neg__(self):
        return _Scaled(-1.0, self)

    def __truediv__(self, other):
        if isinstance(other, _Expr):
            return NotImplemented
        return _Scaled(1.0 / other, self)


class _Prod(_Expr):
    def __init__(self, a, b):
        self.a = a
        self.b = b


class _Sum(_Expr):
    """sum of sign * term"""

    def __init__(self, terms):
        self.terms = []
        for s, t in terms:
            if isinstance(t, _Sum):
                self.terms += [(s * s2, t2) for s2, t2 in t.terms]
            else:
                self.terms.append((s, t))


class _Normal(_Expr):
    """get_normal_vector(Γ): the outward unit normal of a BoundaryTriangulation's facets."""

    def __init__(self, trian):
        self.trian = trian


def get_normal_vector(trian) -> _Normal:
    return _Normal(trian)


class _Basis(_Expr):
    def __init__(self, space, trial: bool, field=None):
        self.space = space
        self.trial = trial
        self.field = field  # position in a MultiFieldFESpace (None: single field)


class _Div(_Expr):
    def __init__(self, arg):
        self.arg = arg


class _Grad(_Expr):
    def __init__(self, arg):
        self.arg = arg


class _Inner(_Expr):
    def __init__(self, a, b):
        self.a = a
        self.b = b


class _Scaled(_Expr):
    def __init__(self, coef, expr):
        self.coef = coef
        self.expr = expr


class _Eps(_Expr):
    def __init__(self, arg):
        self.arg = arg


class _Stress(_Expr):
    def __init__(self, lam, mu, eps):
        self.lam = lam
        self.mu = mu
        self.eps = eps


def symmetric_gradient(a):
    """ε(a) = (∇a + ∇aᵀ)/2 (Fields/DiffOperators.jl:48)."""
    return _Eps(a)


ε = symmetric_gradient


def isotropic_stress(lam, mu):
    """σ(ε) = λ tr(ε) I + 2μ ε, as a function of ε."""
    return lambda e: _Stress(lam, mu, e)


def _multifield(X):
    from .multifield import MultiFieldFESpace
    return isinstance(X, MultiFieldFESpace)


def get_trial_fe_basis(U):
    """The trial basis; on a MultiFieldFESpace one basis per field (a tuple to unpack, as
    Gridap's MultiFieldFEBasis)."""
    if _multifield(U):
        return tuple(_Basis(Ui, True, i) for i, Ui in enumerate(U.spaces))
    return _Basis(U, True)


def get_fe_basis(V):
    if _multifield(V):
        return tuple(_Basis(Vi, False, i) for i, Vi in enumerate(V.spaces))
    return _Basis(V, False)


def divergence(a):
    """∇⋅a of a vector-valued basis (Fields/DiffOperators.jl:7, tr(∇(a)))."""
    return _Div(a)


div = divergence


def gradient(a):
    return _Grad(a)


grad = gradient


def inner(a, b):
    return _Inner(a, b)


dot = inner


class DomainContribution:
    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        return DomainContribution(self.terms + other.terms)


def integrate(expr, measure) -> DomainContribution:
    return DomainContribution([(expr, measure)])


def _strip_scale(e):
    coef = None
    while isinstance(e, _Scaled):
        if coef is not None:
            raise NotImplementedError("nested coefficients")
        coef, e = e.coef, e.expr
    return coef, e


def _elasticity(e):
    if not isinstance(e, _Inner):
        return None
    for x, s in ((e.a, e.b), (e.b, e.a)):
        if isinstance(x, _Eps) and isinstance(s, _Stress) and isinstance(s.eps, _Eps) \
                and isinstance(x.arg, _Basis) and isinstance(s.eps.arg, _Basis) \
                and x.arg.trial != s.eps.arg.trial:
            return s.lam, s.mu
    return None


def classify_bilinear(expr):
    """Returns ("diffusion", coef) for κ ∇v⋅∇u forms and ("elasticity", (λ, μ)) for
    ε(v) ⊙ σ(ε(u)) forms."""
    coef, e = _strip_scale(expr)
    lm = _elasticity(e)
    if lm is not None:
        if coef is not None:
            raise NotImplementedError("scale λ and μ instead of the elasticity form")
        return "elasticity", lm
    if isinstance(e, _Inner):
        ca, a = _strip_scale(e.a)
        cb, b = _strip_scale(e.b)
        if isinstance(a, _Grad) and isinstance(b, _Grad) and isinstance(a.arg, _Basis) \
                and isinstance(b.arg, _Basis) and a.arg.trial != b.arg.trial:
            coefs = [c for c in (coef, ca, cb) if c is not None]
            if len(coefs) > 1:
                raise NotImplementedError("more than one coefficient in the bilinear form")
            return "diffusion", (coefs[0] if coefs else None)
    raise NotImplementedError("bilinear form not recognised (provided: κ*inner(grad(v),grad(u)))")


def classify_linear(expr):
    """Returns ("source", f) for f*v forms and ("body_force", f) for inner(f, v) with a
    constant vector f."""
    if isinstance(expr, _Inner):
        for f, v in ((expr.a, expr.b), (expr.b, expr.a)):
            if isinstance(v, _Basis) and not v.trial and not isinstance(f, _Expr):
                fv = np.asarray(f, dtype=np.float64).reshape(-1)
                if fv.size != 3:
                    raise NotImplementedError("body forces are constant 3-vectors")
                return "body_force", fv
    coef, e = _strip_scale(expr)
    if isinstance(e, _Basis) and not e.trial:
        return "source", (1.0 if coef is None else coef)
    raise NotImplementedError("linear form not recognised (provided: f*v)")


# ---- boundary integrands --------------------------------------------------------------------
BOP_VALUE, BOP_NORMAL_GRAD = 0, 1


def _monomials(e):
    """Expands an integrand into [(factors)]: products of leaves (numbers, callables, bases,
    n⋅∇(basis), n⋅G data) with the signs and constant scales as number factors."""
    if isinstance(e, _Sum):
        out = []
        for s, t in e.terms:
            out += [[s] + m for m in _monomials(t)]
        return out
    if isinstance(e, _Scaled):
        return [[e.coef] + m for m in _monomials(e.expr)]
    if isinstance(e, _Prod):
        return [ma + mb for ma in _monomials(e.a) for mb in _monomials(e.b)]
    return [[e]]


def _normal_grad_of(f):
    """n⋅∇(basis) -> the basis; n⋅G with G a callable -> ('data', G); else None."""
    if not isinstance(f, _Inner):
        return None
    for n, g in ((f.a, f.b), (f.b, f.a)):
        if isinstance(n, _Normal):
            if isinstance(g, _Grad) and isinstance(g.arg, _Basis):
                return g.arg
            if callable(g) and not isinstance(g, _Expr):
                return ("data", g)
    return None


def _split_factor(f):
    """('test'|'trial', op) for a basis factor, ('num', c), ('data', g) or ('ndata', G)."""
    if isinstance(f, _Basis):
        return ("trial" if f.trial else "test", BOP_VALUE)
    ng = _normal_grad_of(f)
    if isinstance(ng, _Basis):
        return ("trial" if ng.trial else "test", BOP_NORMAL_GRAD)
    if isinstance(ng, tuple):
        return ("ndata", ng[1])
    if isinstance(f, (int, float, np.floating, np.integer)):
        return ("num", float(f))
    if callable(f) and not isinstance(f, _Expr):
        return ("data", f)
    raise NotImplementedError(f"boundary integrand factor {type(f).__name__} not recognised")


def classify_boundary_bilinear(expr):
    """Coefficients (c0, c1, c2, c3) of ∫ c0 v u + c1 v (n⋅∇u) + c2 (n⋅∇v) u
    + c3 (n⋅∇v)(n⋅∇u) dΓ."""
    coefs = [0.0, 0.0, 0.0, 0.0]
    for mono in _monomials(expr):
        c, test, trial = 1.0, None, None
        for f in mono:
            kind, val = _split_factor(f)
            if kind == "num":
                c *= val
            elif kind == "test" and test is None:
                test = val
            elif kind == "trial" and trial is None:
                trial = val
            else:
                raise NotImplementedError("boundary bilinear terms carry constant coefficients")
        if test is None or trial is None:
            raise NotImplementedError("each boundary bilinear term needs u and v")
        coefs[2 * test + trial] += c
    return tuple(coefs)


def classify_boundary_linear(expr):
    """[(test_op, scale, data)] of the terms scale * data * op(v): data None (constant), a
    callable g(x), or ('n', G) for n⋅G(x)."""
    out = []
    for mono in _monomials(expr):
        c, test, data = 1.0, None, None
        for f in mono:
            kind, val = _split_factor(f)
            if kind == "num":
                c *= val
            elif kind == "test" and test is None:
                test = val
            elif kind in ("data", "ndata") and data is None:
                data = val if kind == "data" else ("n", val)
            else:
                raise NotImplementedError("boundary linear term not recognised (g v, g n⋅∇v)")
        if test is None:
            raise NotImplementedError("each boundary linear term needs v")
        out.append((test, c, data))
    return out


# ---- quasilinear (nonlinear) integrands ------------------------------------------------------
class _FEState(_Expr):
    """The FE function u a residual or Jacobian is evaluated at (FEOperator's uh)."""

    def __init__(self, fun):
        self.fun = fun


class PowerLawFlux:
    """flux(∇u) = (eps2 + |∇u|²)^((p-2)/2) ∇u — the p-Laplacian flux |∇u|^(p-2) ∇u for
    eps2 = 0 (test/GridapTests/PLaplacianTests.jl). flux(grad(u)) builds the residual's
    integrand factor, flux.derivative(grad(du), grad(u)) the Jacobian's (Gridap's dflux)."""

    def __init__(self, p: float, eps2: float = 0.0):
        self.p = float(p)
        self.eps2 = float(eps2)

    def __call__(self, gradu):
        return _Flux(self, gradu)

    def derivative(self, graddu, gradu):
        return _DFlux(self, graddu, gradu)


class PolynomialCoefficient:
    """α(u) = c0 + c1 u + c2 u² for quasilinear diffusion ∫ α(u) ∇v⋅∇u; α.derivative(u) is
    α'(u) for the Jacobian term ∫ α'(u) du ∇v⋅∇u."""

    def __init__(self, c0: float, c1: float = 0.0, c2: float = 0.0):
        self.c = (float(c0), float(c1), float(c2))

    def __call__(self, u):
        return _Coef(self, u)

    def derivative(self, u):
        return _DCoef(self, u)


class _Flux(_Expr):
    def __init__(self, law, gradu):
        self.law, self.gradu = law, gradu


class _DFlux(_Expr):
    def __init__(self, law, graddu, gradu):
        self.law, self.graddu, self.gradu = law, graddu, gradu


class _Coef(_Expr):
    def __init__(self, law, u):
        self.law, self.u = law, u


class _DCoef(_Expr):
    def __init__(self, law, u):
        self.law, self.u = law, u


def _is_grad_of(e, pred):
    return isinstance(e, _Grad) and pred(e.arg)


def _is_state(e):
    return isinstance(e, _FEState)


def _is_test(e):
    return isinstance(e, _Basis) and not e.trial


def _is_trial(e):
    return isinstance(e, _Basis) and e.trial


def _inner_pair(e, pa, pb):
    """inner(a, b) with pa(a) and pb(b) in either order."""
    if not isinstance(e, _Inner):
        return False
    return (pa(e.a) and pb(e.b)) or (pa(e.b) and pb(e.a))


def _scale_and_rest(mono):
    """Splits a monomial into its numeric scale, per-cell CellFields and other factors."""
    s, cells, rest = 1.0, [], []
    for f in mono:
        if isinstance(f, (int, float, np.floating, np.integer)):
            s *= float(f)
        elif isinstance(f, CellField):
            cells.append(f)
        else:
            rest.append(f)
    return s, cells, rest


class QuasilinearForm:
    """A recognised residual  ∫ κ α(u, ∇u) ∇v⋅∇u - f v  (law, κ, f)."""

    def __init__(self, law, scale, cells, source):
        self.law, self.scale, self.cells, self.source = law, scale, cells, source


def classify_residual(expr) -> QuasilinearForm:
    """Recognises  κ ∇v⋅flux(∇u)  or  κ α(u) ∇v⋅∇u  plus an optional  -f v  term."""
    law = None
    scale, cells, source = 1.0, [], None
    grad_state = lambda e: _is_grad_of(e, _is_state)  # noqa: E731
    grad_test = lambda e: _is_grad_of(e, _is_test)  # noqa: E731
    for mono in _monomials(expr):
        s, cf, rest = _scale_and_rest(mono)
        if len(rest) == 1 and _inner_pair(rest[0], grad_test,
                                          lambda e: isinstance(e, _Flux) and grad_state(e.gradu)):
            lw = rest[0].a.law if isinstance(rest[0].a, _Flux) else rest[0].b.law
        elif len(rest) == 2 and any(isinstance(f, _Coef) and _is_state(f.u) for f in rest) and \
                any(_inner_pair(f, grad_test, grad_state) for f in rest):
            lw = [f for f in rest if isinstance(f, _Coef)][0].law
        elif any(_is_test(f) for f in rest) and not cf:
            data = [f for f in rest if not _is_test(f)]
            if len(rest) - len(data) != 1 or len(data) > 1 or source is not None:
                raise NotImplementedError("one source term f*v is provided in a residual")
            d = data[0] if data else 1.0
            if isinstance(d, _Expr):
                raise NotImplementedError("residual source term not recognised")
            source = (-s, d)  # residual holds -f v: f = -s d
            continue
        else:
            raise NotImplementedError("residual term not recognised (κ ∇v⋅flux(∇u), "
                                      "κ α(u) ∇v⋅∇u, f v)")
        if law is not None:
            raise NotImplementedError("one nonlinear diffusion term is provided")
        law, scale, cells = lw, s, cf
    if law is None:
        raise NotImplementedError("the residual has no nonlinear diffusion term")
    if len(cells) > 1:
        raise NotImplementedError("one per-cell coefficient is provided")
    return QuasilinearForm(law, scale, cells, source)


def check_jacobian(expr, form: QuasilinearForm) -> None:
    """Checks that a user Jacobian is the derivative of the recognised residual's law (the
    device evaluates that derivative exactly); raises NotImplementedError otherwise."""
    grad_state = lambda e: _is_grad_of(e, _is_state)  # noqa: E731
    grad_test = lambda e: _is_grad_of(e, _is_test)  # noqa: E731
    grad_trial = lambda e: _is_grad_of(e, _is_trial)  # noqa: E731
    seen = set()
    for mono in _monomials(expr):
        s, cf, rest = _scale_and_rest(mono)
        same = s == form.scale and [c is k for c, k in zip(cf, form.cells)] == [True] * len(cf) \
            and len(cf) == len(form.cells)
        law = form.law
        if isinstance(law, PowerLawFlux) and len(rest) == 1 and _inner_pair(
                rest[0], grad_test, lambda e: isinstance(e, _DFlux) and e.law is law
                and grad_trial(e.graddu) and grad_state(e.gradu)) and same:
            seen.add("dflux")
        elif isinstance(law, PolynomialCoefficient) and len(rest) == 2 and same and any(
                isinstance(f, _Coef) and f.law is law and _is_state(f.u) for f in rest) and any(
                _inner_pair(f, grad_test, grad_trial) for f in rest):
            seen.add("coef")
        elif isinstance(law, PolynomialCoefficient) and len(rest) == 3 and same and any(
                isinstance(f, _DCoef) and f.law is law and _is_state(f.u) for f in rest) and any(
                _is_trial(f) for f in rest) and any(
                _inner_pair(f, grad_test, grad_state) for f in rest):
            seen.add("dcoef")
        else:
            raise NotImplementedError("the Jacobian is not the derivative of the residual's law")
    need = {"dflux"} if isinstance(form.law, PowerLawFlux) else {"coef", "dcoef"}
    if isinstance(form.law, PolynomialCoefficient) and form.law.c[1] == 0 and \
            form.law.c[2] == 0:
        need = {"coef"}
    if not need <= seen:
        raise NotImplementedError("the Jacobian misses terms of the residual's derivative")


# ---- multi-field integrands -----------------------------------------------------------------
MOP_VALUE, MOP_GRAD, MOP_DIV = 0, 1, 2


class MfTerm:
    """One product term of a multi-field integrand: coef * cell_coef * op_test(v_i) .
    op_trial(u_j) (bilinear) or coef * cell_coef * op_test(v_i) . data (linear, trial_field
    None); data is None (1), a constant (number or sequence) or a callable of x."""

    def __init__(self, test_field, test_op, trial_field, trial_op, coef, cell_coef, data):
        self.test_field, self.test_op = test_field, test_op
        self.trial_field, self.trial_op = trial_field, trial_op
        self.coef, self.cell_coef, self.data = coef, cell_coef, data


def _mf_operand(e):
    """(basis, op) for v, ∇(v) or ∇⋅v; None otherwise."""
    if isinstance(e, _Basis):
        return e, MOP_VALUE
    if isinstance(e, _Grad) and isinstance(e.arg, _Basis):
        return e.arg, MOP_GRAD
    if isinstance(e, _Div) and isinstance(e.arg, _Basis):
        return e.arg, MOP_DIV
    return None


def _mf_expand(e):
    """[(coef, factors)]: the integrand as a sum of products of basis operands, CellFields
    and data, with the numeric scales collected in coef."""
    if isinstance(e, _Sum):
        return [(s * c, f) for s, t in e.terms for c, f in _mf_expand(t)]
    if isinstance(e, _Scaled):
        inner_terms = _mf_expand(e.expr)
        if isinstance(e.coef, (int, float, np.floating, np.integer)):
            return [(float(e.coef) * c, f) for c, f in inner_terms]
        return [(c, [_mf_leaf(e.coef)] + f) for c, f in inner_terms]
    if isinstance(e, (_Prod, _Inner)):
        return [(ca * cb, fa + fb) for ca, fa in _mf_expand(e.a) for cb, fb in _mf_expand(e.b)]
    op = _mf_operand(e)
    if op is not None:
        return [(1.0, [op])]
    if isinstance(e, (int, float, np.floating, np.integer)):
        return [(float(e), [])]
    return [(1.0, [_mf_leaf(e)])]


def _mf_leaf(x):
    if isinstance(x, CellField):
        return x
    if isinstance(x, _Expr):
        raise NotImplementedError(f"multi-field integrand factor {type(x).__name__}")
    if callable(x) or isinstance(x, (tuple, list, np.ndarray)):
        return ("data", x)
    raise NotImplementedError(f"multi-field integrand factor {type(x).__name__}")


def classify_multifield(expr, bilinear: bool):
    """Splits a multi-field integrand into MfTerm products, one test operand each (and one
    trial operand for a bilinear form)."""
    terms = []
    for coef, factors in _mf_expand(expr):
        ops = [f for f in factors if isinstance(f, tuple) and isinstance(f[0], _Basis)]
        cells = [f for f in factors if isinstance(f, CellField)]
        data = [f[1] for f in factors if isinstance(f, tuple) and f[0] == "data"]
        tests = [o for o in ops if not o[0].trial]
        trials = [o for o in ops if o[0].trial]
        if len(tests) != 1 or len(trials) != (1 if bilinear else 0) or len(cells) > 1 \
                or len(data) > (0 if bilinear else 1):
            raise NotImplementedError(
                "each term of a multi-field form is a product of one test operand"
                + (", one trial operand" if bilinear else ", at most one data factor")
                + " and at most one CellField coefficient")
        (vb, vop), = tests
        ub, uop = trials[0] if bilinear else (None, None)
        cell = np.ascontiguousarray(cells[0].values, np.float64) if cells else None
        terms.append(MfTerm(vb.field or 0, vop, None if ub is None else (ub.field or 0), uop,
                            coef, cell, data[0] if data else None))
    return terms
