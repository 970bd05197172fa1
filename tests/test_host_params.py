"""The host mirror of main(params)/hunt(...): parameter defaults and validation as in
GridapMHD src/parameters.jl (no GPU needed: these run before the library is called)."""
import pytest

from gbmhd.main import add_default_params, default_solver_params, hunt
from gbmhd.mesh import hunt_generate_base_mesh


def _params(**over):
    m = hunt_generate_base_mesh((4, 4), Ha=10.0)
    p = {"model": m, "solve": True, "solver": "gb300",
         "fluid": {"domain": None, "α": 1.0, "β": 0.1, "γ": 10.0, "B": (0.0, 1.0, 0.0), "f": (0.0, 0.0, 1.0)},
         "bcs": {"u": {"tags": ["conducting", "insulating"]}, "j": {"tags": "insulating"}}}
    p.update(over)
    return p


def test_defaults_filled():
    """add_default_params (src/parameters.jl:85-137) and params_fluid (:693-723) defaults."""
    p = add_default_params(_params())
    assert p["debug"] is False and p["res_assemble"] is False and p["jac_assemble"] is False
    assert p["check_valid"] is True and p["x0"] == "zero"
    fl = p["fluid"]
    assert fl["σ"] == 1.0 and fl["ζᵤ"] == 0.0 and fl["ζⱼ"] == 0.0 and fl["convection"] == "newton"
    assert p["bcs"]["thin_wall"] == [] and p["bcs"]["φ"] == []
    assert p["fespaces"]["order_u"] == 2 and p["fespaces"]["q"] == 5
    assert p["solver"]["solver"] == "gb300" and p["solver"]["niter"] == 10


def test_ascii_aliases_are_accepted():
    fl = {"domain": None, "alpha": 1.0, "beta": 0.1, "gamma": 10.0, "B": (0.0, 1.0, 0.0), "zeta_u": 2.0}
    p = add_default_params(_params(fluid=fl))
    assert p["fluid"]["α"] == 1.0 and p["fluid"]["ζᵤ"] == 2.0


def test_missing_mandatory_key_message():
    """_check_mandatory (src/parameters.jl:4-14)."""
    p = _params()
    del p["bcs"]
    with pytest.raises(KeyError, match=r"Key :bcs is a mandatory key in params, but it is not provided"):
        add_default_params(p)
    p = _params()
    del p["fluid"]["γ"]
    with pytest.raises(KeyError, match=r"Key :γ is a mandatory key in params\[:fluid\]"):
        add_default_params(p)


def test_invalid_key_message_and_check_valid():
    """_check_unused (src/parameters.jl:47-55): unknown keys fail unless check_valid = false."""
    with pytest.raises(KeyError, match=r"Key :bogus is not a valid key in params\. Set params\[:check_valid\] = false"):
        add_default_params(_params(bogus=1))
    fl = dict(_params()["fluid"], bogus=1)
    with pytest.raises(KeyError, match=r"not a valid key in params\[:fluid\]"):
        add_default_params(_params(fluid=fl))
    p = add_default_params(_params(bogus=1, check_valid=False))
    assert p["bogus"] == 1


def test_thin_wall_entries():
    """params_bcs_thin_wall (src/parameters.jl:938-947): domain, cw and τ mandatory, jw = 0."""
    bcs = {"u": {"tags": ["conducting", "insulating"]}, "j": {"tags": "insulating"},
           "thin_wall": {"domain": "conducting", "cw": 0.1, "τ": 100.0}}
    p = add_default_params(_params(bcs=bcs))
    assert p["bcs"]["thin_wall"] == [{"jw": 0.0, "domain": "conducting", "cw": 0.1, "τ": 100.0}]
    bcs["thin_wall"] = {"domain": "conducting", "cw": 0.1}
    with pytest.raises(KeyError, match=r"Key :τ is a mandatory key in params\[:bcs\]\[:thin_wall\]\[1\]"):
        add_default_params(_params(bcs=bcs))


def test_outside_hot_path_is_refused():
    with pytest.raises(NotImplementedError):
        add_default_params(_params(solid={"domain": "solid", "σ": 1.0}))
    with pytest.raises(NotImplementedError):
        add_default_params(_params(fespaces={"order_u": 3}))
    bcs = {"u": {"tags": ["conducting"]}, "j": {"tags": "insulating"}, "t": [{"tags": "x", "value": 1.0}]}
    with pytest.raises(NotImplementedError, match="tranction"):
        add_default_params(_params(bcs=bcs))
    fl = dict(_params()["fluid"], convection="upwind")
    with pytest.raises(ValueError, match="convection"):
        add_default_params(_params(fluid=fl))


def test_solver_params():
    s = default_solver_params("gb300")
    assert s["precision"] == "mixed" and s["rtol"] == 1e-10 and s["niter_ls"] == 40
    with pytest.raises(ValueError):
        default_solver_params("petsc")
    p = add_default_params(_params(solver={"solver": "gb300", "precision": "fp64", "rtol": 1e-8}))
    assert p["solver"]["precision"] == "fp64" and p["solver"]["rtol"] == 1e-8 and p["solver"]["niter"] == 10
    with pytest.raises(KeyError):
        add_default_params(_params(solver={"precision": "fp64"}))


def test_hunt_keyword_validation():
    """hunt(; kwargs...) (src/Applications/hunt.jl:1-70): unknown keywords and the parts of the
    reference hunt() that are outside this path fail before any device work."""
    with pytest.raises(TypeError, match="unexpected keyword"):
        hunt(nc=(4, 4), bogus=1)
    with pytest.raises(NotImplementedError):
        hunt(nc=(4, 4), tw=0.1)
    with pytest.raises(NotImplementedError):
        hunt(nc=(4, 4), order=3)
    with pytest.raises(ValueError):
        hunt(nc=(4, 4), formulation="other")
