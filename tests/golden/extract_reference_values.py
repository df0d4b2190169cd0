"""Extract the reference's own known answers for the discretize-and-solve path into
reference_values.json (read as text from the dune-gdt source tree; run in a container that has it).

Usage:  python tests/golden/extract_reference_values.py /path/to/dune-gdt
"""
import json
import os
import re
import sys


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def mini_section(text, section):
    out, cur = {}, None
    for line in text.splitlines():
        line = line.split("#")[0].strip()
        if line.startswith("["):
            cur = line.strip("[]")
            continue
        if cur == section and "=" in line:
            k, v = [s.strip() for s in line.split("=", 1)]
            if v.startswith("["):
                out[k] = [float(x) for x in v.strip("[]").split()]
            else:
                try:
                    out[k] = float(v)
                except ValueError:
                    out[k] = v
    return out


def near_triples(text):
    # EXPECT_NEAR((is_simplex_grid_ ? A : B), value, tol)
    pat = re.compile(r"EXPECT_NEAR\(\(is_simplex_grid_ \? ([-0-9.e]+) : ([-0-9.e]+)\), (\w+), ([0-9.e-]+)\)")
    return [(float(a), float(b), name, float(t)) for a, b, name, t in pat.findall(text)]


def main(root):
    res = {}
    lap = "dune/gdt/test/integrands/integrands_laplace.cc"
    prod = "dune/gdt/test/integrands/integrands_product.cc"
    for key, rel in (("q2_stiffness", lap), ("q2_mass", prod)):
        trip = near_triples(read(root, rel))
        res[key] = {
            "source": rel,
            "grid": "[0,3]x[0,1], 9x2 cells (dune/gdt/test/integrands/integrands.hh:64-69), Lagrange order 2",
            "cube": {n: v for (_, v, n, _) in trip},
            "simplex": {n: v for (v, _, n, _) in trip},
            "tolerance": {n: t for (_, _, n, t) in trip},
        }
    burg = "dune/gdt/test/burgers/burgers__1d__explicit__fv.mini"
    text = read(root, burg)
    res["burgers_1d"] = {"source": burg}
    for flux in ("numerical_upwind_flux", "numerical_lax_friedrichs_flux", "numerical_engquist_osher_flux"):
        base = "Burgers1dExplicitFvTest.periodic_boundaries__" + flux
        res["burgers_1d"][flux] = {"setup": mini_section(text, base + ".setup"),
                                   "results": mini_section(text, base + ".results")}
    esv = "dune/gdt/test/stationary-heat-equation/stationary_heat_equation__ESV2007__table_1.mini"
    res["esv2007_cube"] = {"source": esv,
                           "results": mini_section(read(root, esv),
                                                   "NearlyESV2007Table1ButWithCubicGridTest.columns_1_to_5.results")}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_values.json")
    with open(out, "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract_reference_values.py <root of the dune-gdt source tree>")
    main(sys.argv[1])
