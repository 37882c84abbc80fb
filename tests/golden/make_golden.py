"""Extract the reference's element-level golden vectors into JSON fixtures.

The reference keeps its known-answer vectors as literal arrays inside its unit
tests.  This script reads those test files AS TEXT (Python ``ast``; nothing of
the reference is imported or executed) and writes one JSON fixture per test
file into this directory.  Each array records the ``file:line`` it came from.

Run it where the reference checkout is present::

    python tests/golden/make_golden.py <path of the folax checkout>

The fixtures are committed; nothing at test time reads the reference.
"""
import ast
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _arrays_by_function(path):
    """Return {function_name: [(lineno, ndarray), ...]} for literal jnp.array calls."""
    tree = ast.parse(open(path).read())
    out = {}
    for node in ast.walk(tree):
        if not isinstance(node, ast.FunctionDef):
            continue
        arrs = []
        for sub in ast.walk(node):
            if (isinstance(sub, ast.Call) and getattr(sub.func, "attr", None) == "array"
                    and sub.args):
                try:
                    val = ast.literal_eval(sub.args[0])
                except ValueError:
                    continue
                arrs.append((sub.lineno, np.asarray(val, dtype=np.float64)))
        arrs.sort(key=lambda t: t[0])
        out[node.name] = arrs
    return out


def _entry(rel, lineno, arr):
    return {"src": f"{rel}:{lineno}", "shape": list(arr.shape),
            "data": arr.ravel().tolist()}


def element_tests(ref_root, rel):
    """K_e / r_e goldens for tet4, hex8, quad4 (E=1, nu=0.3, controls=1, u=1)."""
    fns = _arrays_by_function(os.path.join(ref_root, rel))
    out = {}
    for fn, key in (("test_tetra", "tet4"), ("test_hexa", "hex8"), ("test_quad", "quad4")):
        arrs = fns[fn]
        by_shape = {}
        # order in the source: coordinates, [body force], stiffness, residual
        coords = arrs[0]
        body = [a for a in arrs if a[1].ndim == 2 and a[1].shape[1] == 1]
        mats = [a for a in arrs if a[1].ndim == 2 and a[1].shape[0] == a[1].shape[1]
                and a[1].shape[0] > 4]
        vecs = [a for a in arrs if a[1].ndim == 1]
        by_shape["xyz"] = _entry(rel, *coords)
        by_shape["body_force"] = _entry(rel, *body[0])
        by_shape["stiffness"] = _entry(rel, *mats[0])
        by_shape["residual"] = _entry(rel, *vecs[0])
        by_shape["young_modulus"] = 1.0
        by_shape["poisson_ratio"] = 0.3
        by_shape["rtol"] = 1e-5
        by_shape["atol"] = 1e-6
        out[key] = by_shape
    return out


def geometry_tests(ref_root):
    rel = "tests/unit/test_geometries.py"
    fns = _arrays_by_function(os.path.join(ref_root, rel))
    setup = fns["setUp"]
    coords = {"quad4": setup[1], "tet4": setup[2], "hex8": setup[3]}
    out = {}
    q = fns["test_quad2D4"]
    out["quad4"] = {
        "xyz": _entry(rel, *coords["quad4"]),
        "gi1": {"points": _entry(rel, *q[0]), "weights": _entry(rel, *q[1]),
                "N": _entry(rel, *q[2]), "dN_dxi": _entry(rel, *q[3]),
                "jacobian": _entry(rel, *q[4]), "dN_dx": _entry(rel, *q[5])},
        "gi2": {"points": _entry(rel, *q[6]), "weights": _entry(rel, *q[7])},
        "gi3": {"points": _entry(rel, *q[8]), "weights": _entry(rel, *q[9])},
    }
    t = fns["test_tet3D4"]
    out["tet4"] = {
        "xyz": _entry(rel, *coords["tet4"]),
        "gi1": {"points": _entry(rel, *t[0]), "weights": _entry(rel, *t[1]),
                "N": _entry(rel, *t[2]), "dN_dxi": _entry(rel, *t[3]),
                "jacobian": _entry(rel, *t[4]), "dN_dx": _entry(rel, *t[5])},
        "gi2": {"points": _entry(rel, *t[6]), "weights": _entry(rel, *t[7]),
                "N": _entry(rel, *t[8]), "dN_dxi": _entry(rel, *t[9]),
                "jacobian": _entry(rel, *t[10]), "dN_dx": _entry(rel, *t[11])},
        "gi3": {"points": _entry(rel, *t[12]), "weights": _entry(rel, *t[13])},
    }
    h = fns["test_hex3D8"]
    out["hex8"] = {
        "xyz": _entry(rel, *coords["hex8"]),
        "gi1": {"points": _entry(rel, *h[0]), "weights": _entry(rel, *h[1]),
                "N": _entry(rel, *h[2]), "dN_dxi": _entry(rel, *h[3]),
                "jacobian": _entry(rel, *h[4]), "dN_dx": _entry(rel, *h[5])},
        "gi2": {"points": _entry(rel, *h[6]), "weights": _entry(rel, *h[7])},
        "gi3": {"points": _entry(rel, *h[8]), "weights": _entry(rel, *h[9])},
    }
    out["rtol"] = 1e-5
    out["atol"] = 1e-6
    return out


def sensitivity_test(ref_root):
    rel = "tests/unit/test_sensitivity_analysis.py"
    fns = _arrays_by_function(os.path.join(ref_root, rel))
    arrs = [a for a in fns["test_quad"]]
    # source order (by line): u(18) K(9) [freqs] jac_row(18) rhs(18) adj_u(18) dctrl(9) dshape(27)
    by_line = {ln: a for ln, a in arrs}
    lines = sorted(by_line)
    big = [(ln, by_line[ln]) for ln in lines if by_line[ln].size >= 9]
    names = ["u", "control", "jacobian_row8", "rhs", "adjoint_u",
             "control_derivatives", "shape_derivatives"]
    assert len(big) == len(names), [b[1].shape for b in big]
    out = {n: _entry(rel, *b) for n, b in zip(names, big)}
    out.update({"mesh_N": 3, "mesh_L": 1.0, "young_modulus": 1.0, "poisson_ratio": 0.3,
                "num_gp": 2,
                "bc": {"Ux": {"left": 0.0, "right": 0.05}, "Uy": {"left": 0.0, "right": 0.05}},
                "response_formula": "(E**2)*U[0]", "rtol": 1e-5, "atol": 1e-5})
    return out


def transient_thermal_tests(ref_root):
    """Implicit-Euler transient thermal element (test_nonlinear_transient_thermal.py):
    T_current = 1, T_next = 0, k0 = 1, rho = cp = 1, beta = 1.5, c = 1, dt = 0.005."""
    rel = "tests/unit/test_nonlinear_transient_thermal.py"
    fns = _arrays_by_function(os.path.join(ref_root, rel))
    out = {}
    for fn, key in (("test_tetra", "tet4"), ("test_hexa", "hex8")):
        arrs = fns[fn]
        coords = arrs[0]
        mats = [a for a in arrs if a[1].ndim == 2 and a[1].shape[0] == a[1].shape[1] and a[1].shape[0] > 3]
        vecs = [a for a in arrs if a[1].ndim == 1 and a[1].size > 3]
        out[key] = {"xyz": _entry(rel, *coords), "stiffness": _entry(rel, *mats[0]),
                    "residual": _entry(rel, *vecs[0])}
    out.update({"rho": 1.0, "cp": 1.0, "beta": 1.5, "c": 1.0, "time_step": 0.005, "rtol": 1e-5, "atol": 1e-10})
    return out


def mesh_io_tests(ref_root):
    """The .mdpa fixture of tests/unit/test_mesh_io.py (copied next to this
    script) and the counts that test asserts for it (read as text)."""
    import re
    import shutil
    rel = "tests/unit/test_mesh_io.py"
    text = open(os.path.join(ref_root, rel)).read()
    src = lambda m: f"{rel}:{text.count(chr(10), 0, m.start()) + 1}"  # noqa: E731
    out = {"file": "coarse_sphere.mdpa", "node_sets": {}}
    m = re.search(r"self\.mdpa_io\.GetNumberOfNodes\(\),\s*(\d+)", text)
    out["num_nodes"] = {"value": int(m.group(1)), "src": src(m)}
    m = re.search(r'self\.mdpa_io\.GetNumberOfElements\("(\w+)"\),\s*(\d+)', text)
    out["num_elements"] = {"type": m.group(1), "value": int(m.group(2)), "src": src(m)}
    for m in re.finditer(r'len\(self\.mdpa_io\.GetNodeSet\("(\w+)"\)\),\s*(\d+)', text):
        out["node_sets"][m.group(1)] = {"value": int(m.group(2)), "src": src(m)}
    shutil.copyfile(os.path.join(ref_root, "tests/meshes/coarse_sphere.mdpa"), os.path.join(HERE, "coarse_sphere.mdpa"))
    return out


def main(ref_root):
    fixtures = {
        "mesh_io.json": mesh_io_tests(ref_root),
        "mechanical_linear.json": element_tests(ref_root, "tests/unit/test_mechanical_loss.py"),
        "neohooke_ad.json": element_tests(ref_root, "tests/unit/test_neo_hooke_mechanical_loss_AD.py"),
        "neohooke.json": element_tests(ref_root, "tests/unit/test_neo_hooke_mechanical_loss.py"),
        "geometries.json": geometry_tests(ref_root),
        "sensitivity_quad4.json": sensitivity_test(ref_root),
        "transient_thermal.json": transient_thermal_tests(ref_root),
    }
    for name, obj in fixtures.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the folax checkout>")
    main(sys.argv[1])
