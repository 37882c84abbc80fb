"""Response formula parsing (CPU): the reference's formula strings
(fe_response.py:58-62) become the monomials the response kernel evaluates."""
import pytest

from folax_gb300.response import parse_response_formula


def _as_dict(monos):
    return {(p, q): c for c, p, q in monos}


def test_reference_formula():
    assert _as_dict(parse_response_formula("(E**2)*U[0]", "E", "U", 2)) == {(2, (1, 0, 0)): 1.0}


def test_expansion_and_constants():
    got = _as_dict(parse_response_formula("0.5*(U[0] + E*U[1])**2 - 3*E/2 + 1", "E", "U", 3))
    assert got == {(0, (2, 0, 0)): 0.5, (1, (1, 1, 0)): 1.0, (2, (0, 2, 0)): 0.5, (1, (0, 0, 0)): -1.5,
                   (0, (0, 0, 0)): 1.0}


def test_thermal_name_and_cancellation():
    assert _as_dict(parse_response_formula("K*T[0] - T[0]*K + T[0]**3", "K", "T", 1)) == {(0, (3, 0, 0)): 1.0}


@pytest.mark.parametrize("bad", ["jnp.sin(E)", "E**0.5", "U[3]", "E/U[0]", "X*U[0]", "E**U[0]"])
def test_unsupported_formulas_raise(bad):
    with pytest.raises(NotImplementedError):
        parse_response_formula(bad, "E", "U", 3)
