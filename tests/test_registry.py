"""The integrator registry keeps the reference's contract (quad/_registry.py, quad/__init__.py)."""

import warnings

import pytest

from braincell_gb300 import quad
from braincell_gb300.quad import IntegratorRegistry, get_integrator


def test_gb300_step_registered_with_aliases():
    f = get_integrator("gb300_staggered")
    assert f is quad.gb300_staggered_step
    assert get_integrator("gb300") is f and get_integrator("staggered_gb300") is f
    e = quad.get_registry().entry("gb300")
    assert e.name == "gb300_staggered" and e.category == "staggered"
    assert "gb300_staggered" in quad.all_integrators and "gb300" in quad.all_integrators


def test_unknown_name_suggests():
    with pytest.raises(ValueError, match="Did you mean 'gb300_staggered'"):
        get_integrator("gb300_staggerd")


def test_callable_passthrough_and_type_error():
    def f(target):
        return None

    assert get_integrator(f) is f
    with pytest.raises(TypeError):
        get_integrator(3)


def test_register_collisions_and_override():
    r = IntegratorRegistry()

    def a(t):
        pass

    def b(t):
        pass

    r.register("euler", a, aliases=("explicit",), category="explicit", order=1)
    assert r["explicit"] is a and r.resolve("explicit") == "euler"
    with pytest.raises(ValueError):
        r.register("euler", b)
    with pytest.raises(ValueError):
        r.register("explicit", b)
    with pytest.raises(ValueError):
        r.register("other", b, aliases=("explicit",))
    with pytest.warns(RuntimeWarning):
        r.register("euler", b, override=True)
    assert r["euler"] is b and "explicit" not in r
    with pytest.raises(TypeError):
        r.register("", a)
    with pytest.raises(TypeError):
        r.register("x", 3)
    with pytest.raises(TypeError):
        r.register("y", a, aliases=("",))


def test_deprecated_warns_once_and_unregister():
    r = IntegratorRegistry()

    def a(t):
        pass

    r.register("old", a, deprecated=True)
    with pytest.warns(DeprecationWarning):
        r.entry("old")
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        r.entry("old")
    r.unregister("old")
    assert "old" not in r and len(r) == 0
    with pytest.raises(KeyError):
        r.unregister("old")


def test_names_categories_dict():
    r = IntegratorRegistry()

    def a(t):
        pass

    def b(t):
        pass

    r.register("b_step", b, aliases=("bb",), category="voltage")
    r.register("a_step", a, category="voltage")
    assert r.names() == ["a_step", "b_step"]
    assert r.names(include_aliases=True) == ["a_step", "b_step", "bb"]
    assert [e.name for e in r.by_category("voltage")] == ["a_step", "b_step"]
    assert set(r.as_dict()) == {"a_step", "b_step", "bb"}
    assert r.get("missing") is None


def test_step_rejects_non_cell_target():
    with pytest.raises(TypeError):
        quad.gb300_staggered_step(object())
