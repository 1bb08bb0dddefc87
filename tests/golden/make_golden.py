"""Extract the reference's own known-answer vectors for the hot path into
``tests/golden/reference_unit_vectors.json``.

The reference (smillerc/fvleg_2d) is Fortran with no compiler in this environment, so its unit
tests are read as text:

* ``tests/unit/make_simple_grid.py``             -- the 4x4 ``simple.h5`` interior values;
* ``tests/unit/test_bc/mod_test_bc.f90``         -- single-image asserts of the periodic,
  symmetry and zero-gradient boundary conditions (which BCs are applied, in which order);
* ``tests/unit/test_limiters/test_limiters.f90`` -- flux-limiter values;
* ``tests/unit/test_reconstruction/test_reconstruction.pf`` -- TVD2 edge values;
* ``tests/unit/test_geometry/test_quad_cell.pf`` and ``mod_test_grid.f90`` -- cell metrics and
  the simple grid's node coordinates;
* ``tests/unit/test_field/test_field.f90`` -- the halo exchange of an 8x8 field over 2x2 images
  (``sync_edges``): each image's interior values and the halo rows it receives across j.

It also copies the reference's one HDF5 file, ``tests/unit/simple.h5`` (written by
``make_simple_grid.py`` through h5py: gzip-compressed chunks, variable-length string
attributes), byte for byte to ``tests/golden/reference_simple.h5``: the known-answer input of the
HDF5 reader (``fvleg_2d_gb300/h5lite.py``).

Run from the repository root with the environment variable REFERENCE naming the reference
checkout:  ``REFERENCE=<checkout> python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys

REF = os.environ.get("REFERENCE", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_unit_vectors.json")

NUM = r"[-+]?\d+\.\d*(?:_rk)?"


def read(rel: str) -> str:
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def nums(s: str) -> list[float]:
    return [float(x.replace("_rk", "")) for x in re.findall(NUM, s)]


def simple_grid() -> dict:
    """Interior rows of simple.h5 from make_simple_grid.py: data[2:6, j] = [..] (j = python
    index incl. 2 ghost layers)."""
    src = read("tests/unit/make_simple_grid.py")
    rows = {}
    for m in re.finditer(r"data\[2:6,\s*(\d+)\]\s*=\s*\[([^\]]*)\]", src):
        rows[int(m.group(1)) - 2 + 1] = [float(x) for x in m.group(2).split(",")]
    # reference (i, j), 1-based interior j -> values for i = 1..4
    m = re.search(r"make_uniform_grid\(n_cells=\((\d+),\s*(\d+)\),\s*xrange=\(([-\d.]+),\s*([-\d.]+)\),"
                  r"\s*yrange=\(([-\d.]+),\s*([-\d.]+)\),\s*n_ghost_layers=(\d+)", src)
    ni, nj, x0, x1, y0, y1, ng = m.groups()
    return {"ni": int(ni), "nj": int(nj), "n_ghost": int(ng), "xrange": [float(x0), float(x1)],
            "yrange": [float(y0), float(y1)], "rows": {str(k): v for k, v in sorted(rows.items())},
            "source": "tests/unit/make_simple_grid.py"}


def bc_cases() -> list[dict]:
    """Single-image (num_images() == 1) asserts of each BC test subroutine."""
    src = read("tests/unit/test_bc/mod_test_bc.f90")
    lines = src.splitlines()
    cases = []
    i = 0
    while i < len(lines):
        m = re.match(r"\s*subroutine (test_\w+)\(\)", lines[i])
        if not m or m.group(1) == "test_pressure":
            i += 1
            continue
        name, start = m.group(1), i + 1
        body = []
        i += 1
        while not re.match(r"\s*end subroutine", lines[i]):
            body.append((i + 1, lines[i]))
            i += 1
        factory = {}
        applied = []
        single = []
        depth = 0
        in_single = False
        arrays = {}
        for ln, text in body:
            code = text.split("!")[0]
            fm = re.search(r"(bc_\w+)\s*=>\s*bc_factory\(bc_type='(\w+)',\s*location='([+-][xy])'", code)
            if fm:
                factory[fm.group(1)] = (fm.group(2), fm.group(3))
            am = re.search(r"call (bc_\w+)%apply\(", code)
            if am:
                applied.append(factory[am.group(1)])
            if re.search(r"select case\s*\(num_images\(\)\)", code):
                depth = 1
                continue
            if depth >= 1 and re.search(r"select case", code):
                depth += 1
                continue
            if depth >= 1 and re.search(r"end select", code):
                depth -= 1
                if depth == 0:
                    in_single = False
                continue
            if depth == 1 and re.match(r"\s*case\s*\(1\)", code):
                in_single = True
                continue
            if depth == 1 and re.match(r"\s*case", code):
                in_single = False
                continue
            if not in_single:
                continue
            vm = re.match(r"\s*(\w+)\s*=\s*\[(.*)\]\s*$", code)
            if vm:
                arrays[vm.group(1)] = nums(vm.group(2))
                continue
            cm = re.search(r"assert_equal\(\s*(-?)\s*(\[[^\]]*\]|\w+)\s*,\s*(\w+)%data\(([^)]*)\)", code)
            if cm:
                neg, expr, field, index = cm.groups()
                vals = nums(expr) if expr.startswith("[") else list(arrays[expr])
                if neg:
                    vals = [-v for v in vals]
                single.append({"field": field, "index": [s.strip() for s in index.split(",")],
                               "expected": vals, "line": ln})
        cases.append({"test": name, "line": start, "applied": applied, "checks": single})
    return cases


def limiter_values() -> dict:
    src = read("tests/unit/test_limiters/test_limiters.f90")
    out = {}
    name = None
    for line in src.splitlines():
        m = re.search(r"flux_limiter_t\(name='(\w+)'\)", line)
        if m:
            name = m.group(1)
            out[name] = []
        m = re.search(r"assert_equal\(\s*(" + NUM + r")\s*,\s*limiter%limit\(\s*(" + NUM + r")\s*\)", line)
        if m and name:
            out[name].append([float(m.group(2).replace("_rk", "")), float(m.group(1).replace("_rk", ""))])
    return {"values": out, "source": "tests/unit/test_limiters/test_limiters.f90"}


def tvd2_none() -> dict:
    src = read("tests/unit/test_reconstruction/test_reconstruction.pf")
    seg = src[src.index("subroutine test_tvd2_none"):src.index("endsubroutine test_tvd2_none")]
    cols = {int(m.group(1)): float(m.group(2).replace("_rk", ""))
            for m in re.finditer(r"rho\((-?\d+),\s*:\)\s*=\s*(" + NUM + ")", seg)}
    asserts = [[int(m.group(2)), float(m.group(1).replace("_rk", ""))]
               for m in re.finditer(r"@assertEqual\((" + NUM + r"),\s*edge_vars\((\d),\s*i,\s*j\)\)", seg)]
    ij = re.search(r"i = (\d+)\s*\n\s*j = (\d+)\s*\n\s*@assert", seg)
    return {"column_values": {str(k): v for k, v in sorted(cols.items())},
            "cell": [int(ij.group(1)), int(ij.group(2))], "edge_values": asserts,
            "edge_numbering": "1 bottom, 2 right, 3 top, 4 left (cell-based, old API)",
            "source": "tests/unit/test_reconstruction/test_reconstruction.pf"}


def quad_cell() -> dict:
    src = read("tests/unit/test_geometry/test_quad_cell.pf")
    x = nums(re.search(r"dimension\(4\) :: x = \[([^\]]*)\]", src).group(1))
    y = nums(re.search(r"dimension\(4\) :: y = \[([^\]]*)\]", src).group(1))
    vol = float(re.search(r"@assertEqual\(([\d.]+),\s*cell%volume\)", src).group(1))
    el = [float(m.group(1).replace("_rk", "")) for m in
          re.finditer(r"@assertEqual\((" + NUM + r"),\s*cell%edge_lengths\(\d\)\)", src)]
    nv = [nums(m.group(1)) for m in
          re.finditer(r"@assertEqual\(\[([^\]]*)\],\s*cell%edge_norm_vectors\(:,\s*\d\)\)", src)]
    return {"x": x, "y": y, "volume": vol, "edge_lengths": el, "edge_norm_vectors": nv,
            "source": "tests/unit/test_geometry/test_quad_cell.pf"}


def grid_nodes() -> dict:
    src = read("tests/unit/test_geometry/mod_test_grid.f90")
    seg = src[src.index("! Single-image testing is a bit easier"):]
    x = nums(re.search(r"assert_equal\(\[([^\]]*)\],\s*&?\s*grid%node_x", seg, re.S).group(1))
    y = {int(m.group(2)): float(m.group(1).replace("_rk", "")) for m in
         re.finditer(r"assert_equal\((" + NUM + r"),\s*grid%node_y\(:,\s*(-?\d+)\)", seg)}
    return {"node_x": x, "node_y": {str(k): v for k, v in sorted(y.items())},
            "source": "tests/unit/test_geometry/mod_test_grid.f90"}


def field_halo() -> dict:
    """test_halo_exchange: per image (1..4) its interior rows ``field%data(a:b, j) = [..]`` and
    the asserted halo rows ``field%data(ilo_halo:ihi_halo, jhi_halo[ - 1])`` /
    ``(.., jlo_halo[ + 1])`` (a scalar 0.0 assert is a row of zeros)."""
    src = read("tests/unit/test_field/test_field.f90")
    body = src[src.index("subroutine test_halo_exchange"):src.index("end subroutine test_halo_exchange")]
    setup, checks = body.split("call field%sync_edges()")
    images = {}
    parts = re.split(r"case\((\d)\)", setup)
    for k in range(1, len(parts), 2):
        img = int(parts[k])
        rows = {}
        for a, b, j, vals in re.findall(r"field%data\((\d+):(\d+),\s*(\d+)\)\s*=\s*\[([^\]]*)\]",
                                        parts[k + 1]):
            rows[j] = {"i0": int(a), "i1": int(b), "values": nums(vals)}
        images[str(img)] = {"rows": rows}
    parts = re.split(r"case\((\d)\)", checks)
    for k in range(1, len(parts), 2):
        img = str(int(parts[k]))
        halo = {}
        pat = (r"call assert_equal\((\[[^\]]*\]|0\.0_rk),\s*&?\s*"
               r"field%data\(ilo_halo:ihi_halo,\s*(j(?:hi|lo)_halo(?:\s*[-+]\s*1)?)\)")
        for vals, where in re.findall(pat, parts[k + 1]):
            key = where.replace(" ", "")
            halo[key] = nums(vals) if vals.startswith("[") else [0.0] * 8
        images[img]["halo_rows"] = halo
    return {"ni": 8, "nj": 8, "n_halo": 2, "images": images,
            "source": "tests/unit/test_field/test_field.f90 (test_halo_exchange)"}


def main() -> int:
    if not REF or not os.path.isdir(REF):
        print("set REFERENCE to the reference checkout", file=sys.stderr)
        return 2
    data = {
        "generated_by": "tests/golden/make_golden.py",
        "reference": "smillerc/fvleg_2d",
        "simple_grid": simple_grid(),
        "bc": {"source": "tests/unit/test_bc/mod_test_bc.f90", "cases": bc_cases()},
        "limiters": limiter_values(),
        "tvd2_none": tvd2_none(),
        "quad_cell": quad_cell(),
        "grid_nodes": grid_nodes(),
        "field_halo": field_halo(),
    }
    n_checks = sum(len(c["checks"]) for c in data["bc"]["cases"])
    if n_checks < 40:
        print(f"too few BC asserts extracted ({n_checks})", file=sys.stderr)
        return 1
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    h5 = os.path.join(os.path.dirname(OUT), "reference_simple.h5")
    shutil.copyfile(os.path.join(REF, "tests", "unit", "simple.h5"), h5)
    print(f"wrote {OUT}: {len(data['bc']['cases'])} BC tests, {n_checks} asserts; {h5}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
