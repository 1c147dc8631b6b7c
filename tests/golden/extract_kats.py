"""Extracts known-answer values from Gridap.jl's own test suite into gridap_kats.json.

Gridap is Julia and cannot run here, so its test files are read as text: the literal
arrays and numbers in the assertions listed below become the golden vectors that pin the
oracle (and, through it, the GPU library). Run from the repository root:

    python tests/golden/extract_kats.py /path/to/Gridap.jl

Each entry records the file and line it came from.
"""
from __future__ import annotations

import json
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent


def julia_array(text: str):
    """Parses a Julia array literal of ints/floats/tuples (VectorValue{..}[(a,b),...] too)."""
    t = re.sub(r"^[A-Za-z_][A-Za-z0-9_{}, ]*\[", "[", text.strip())
    t = t.replace("(", "[").replace(")", "]")
    return json.loads(t)


def find(lines, pattern, start=0):
    rx = re.compile(pattern)
    for i in range(start, len(lines)):
        if rx.search(lines[i]):
            return i
    raise LookupError(pattern)


def rhs_after(line: str, op: str) -> str:
    return line.split(op, 1)[1].strip()


def collect_bracketed(lines, i, opener):
    """Text from the first `opener` on line i to its matching close bracket (multi-line)."""
    s = lines[i][lines[i].index(opener):]
    depth = 0
    out = []
    j = i
    while True:
        for ch in s:
            out.append(ch)
            if ch == "[":
                depth += 1
            elif ch == "]":
                depth -= 1
                if depth == 0:
                    return "".join(out), j
        j += 1
        s = lines[j]


def main(ref: pathlib.Path):
    kats = {}

    # ---- assembled 2x2 Poisson (SparseMatrixAssemblersTests.jl) ---------------------------
    f = "test/FESpacesTests/SparseMatrixAssemblersTests.jl"
    L = (ref / f).read_text().splitlines()
    i_tags = find(L, r"V = FESpace\(model,reffe,dirichlet_tags=")
    tags = julia_array(L[i_tags].split("dirichlet_tags=")[1].rstrip(")"))
    i_vec = find(L, r"@test vec ≈ \[")
    vec = julia_array(rhs_after(L[i_vec], "≈"))
    entries = []
    j = i_vec + 1
    while "@test mat[" in L[j]:
        m = re.search(r"mat\[(\d+),\s*(\d+)\]\s*≈\s*([-0-9.eE]+)", L[j])
        entries.append([int(m.group(1)), int(m.group(2)), float(m.group(3)), j + 1])
        j += 1
    kats["poisson_2x2_q1"] = {
        "source": f"{f}:{i_tags + 1},{i_vec + 1}-{j}",
        "domain": [0, 1, 0, 1], "partition": [2, 2], "order": 1, "degree": 2,
        "dirichlet_tags": tags, "f": "x[2]",
        "vec": vec, "mat_entries": [e[:3] for e in entries],
        "note": "Julia ≈ (rtol sqrt(eps)); values printed with ~15 digits",
    }

    # ---- CLagrangian numbering (CLagrangianFESpacesTests.jl) ------------------------------
    f = "test/FESpacesTests/CLagrangianFESpacesTests.jl"
    L = (ref / f).read_text().splitlines()
    kl = {}
    i = find(L, r"V = CLagrangianFESpace\(VectorValue\{2,Float64\},grid\)")
    i = find(L, r"@test get_cell_dof_ids\(V\) ==", i)
    kl["vector_cell_dofs"] = julia_array(rhs_after(L[i], "=="))
    kl["vector_cell_dofs_line"] = i + 1
    i = find(L, r"V.metadata.node_and_comp_to_dof ==", i)
    kl["vector_node_and_comp_to_dof"] = julia_array(rhs_after(L[i], "=="))
    i = find(L, r"^tags = \[")
    kl["tags"] = julia_array(rhs_after(L[i], "="))
    i = find(L, r"^masks1 = ")
    kl["masks1"] = [bool(x) for x in julia_array(rhs_after(L[i], "=").replace("Bool", "")
                                                  .replace("true", "1").replace("false", "0"))]
    i = find(L, r"@test get_cell_dof_ids\(V\) ==", i)
    kl["masked_cell_dofs"] = julia_array(rhs_after(L[i], "=="))
    kl["masked_cell_dofs_line"] = i + 1
    i = find(L, r"V.metadata.free_dof_to_node ==", i)
    kl["masked_free_dof_to_node"] = julia_array(rhs_after(L[i], "=="))
    i = find(L, r"V.metadata.dirichlet_dof_to_node ==", i)
    kl["masked_dirichlet_dof_to_node"] = julia_array(rhs_after(L[i], "=="))
    i = find(L, r"V.metadata.node_and_comp_to_dof ==", i)
    kl["masked_node_and_comp_to_dof"] = julia_array(rhs_after(L[i], "=="))
    i = find(L, r"^masks2 = ")
    m2 = rhs_after(L[i], "=").replace("true", "1").replace("false", "0")
    kl["masks2"] = [[bool(v) for v in t] for t in julia_array(m2)]
    i = find(L, r"@test get_cell_dof_ids\(V\) ==", i)
    kl["masked_vector_cell_dofs"] = julia_array(rhs_after(L[i], "=="))
    i = find(L, r"V.metadata.node_and_comp_to_dof ==", i)
    kl["masked_vector_node_and_comp_to_dof"] = julia_array(rhs_after(L[i], "=="))
    kl["source"] = f
    kl["domain"] = [0, 1, 0, 1]
    kl["partition"] = [2, 2]
    kats["clagrangian_2x2"] = kl

    # ---- QUAD edge/vertex tables (ExtrusionPolytopesTests.jl) -----------------------------
    f = "test/ReferenceFEsTests/ExtrusionPolytopesTests.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"@test get_faces\(p,1,0\) ==")
    kats["quad_edge_vertices"] = {"source": f"{f}:{i + 1}",
                                  "value": julia_array(rhs_after(L[i], "=="))}
    i = find(L, r"@test get_facedims\(p\) ==")
    kats["quad_facedims"] = {"source": f"{f}:{i + 1}", "value": julia_array(rhs_after(L[i], "=="))}

    # ---- quadrature exactness (TensorProductQuadraturesTests.jl) --------------------------
    f = "test/ReferenceFEsTests/TensorProductQuadraturesTests.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"for degree in 1:10")
    j = find(L, r"@test err < ", i)
    kats["tensor_quadrature_exactness"] = {
        "source": f"{f}:{i + 1}-{j + 1}", "degrees": [1, 10], "polytopes": ["QUAD", "HEX"],
        "max_rel_err": float(re.search(r"err < ([0-9.eE+-]+)", L[j]).group(1)),
        "note": "monomials x^a y^b (z^c) with each exponent <= degree integrate to 1/prod(a+1)",
    }

    # ---- conforming Q2 numbering on 3x3 quads (ConformingFESpacesTests.jl) -----------------
    f = "test/FESpacesTests/ConformingFESpacesTests.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"^dirichlet_tags = ")
    dtags = julia_array(rhs_after(L[i], "=").replace('"', '"'))
    i = find(L, r"^r = \[", i)
    txt, j = collect_bracketed(L, i, "[")
    r_q2 = julia_array(txt)
    i2 = find(L, r"@test nfree == ", j)
    nfree = int(rhs_after(L[i2], "=="))
    i3 = find(L, r"@test ndiri == ", j)
    ndiri = int(rhs_after(L[i3], "=="))
    kats["conforming_q2_3x3"] = {"source": f"{f}:{i + 1}-{i3 + 1}", "domain": [0, 1, 0, 1],
                                 "partition": [3, 3], "order": 2, "dirichlet_tags": dtags,
                                 "cell_dofs": r_q2, "nfree": nfree, "ndiri": ndiri}

    # ---- simplexify(HEX) local tets (ExtrusionPolytopes.jl source) -------------------------
    f = "src/ReferenceFEs/ExtrusionPolytopes.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"^function oriented_simplexify_hypercube")
    i = find(L, r"elseif dim == 3", i)
    txt, j = collect_bracketed(L, i + 1, "[")
    kats["hex_simplexify"] = {"source": f"{f}:{i + 2}-{j + 1}", "tets": julia_array(txt)}
    f = "test/ReferenceFEsTests/ExtrusionPolytopesTests.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"p = Polytope\(TET_AXIS, TET_AXIS, TET_AXIS\)")
    i = find(L, r"^x = Point\{3,Float64\}\[", i)
    kats["tet_vertex_coordinates"] = {"source": f"{f}:{i + 1}",
                                      "value": julia_array(rhs_after(L[i], "="))}

    # ---- Witherden-Vincent tet rule for degrees 4 and 5 (source tables) --------------------
    f = "src/ReferenceFEs/WitherdenVincentQuadratures.jl"
    L = (ref / f).read_text().splitlines()
    i0 = find(L, r"^function _witherdenvincent_quad_tet")
    i = find(L, r"elseif degree in \(4, 5\)", i0)
    tx2, j2 = collect_bracketed(L, find(L, r"data2 = \[", i), "[")
    tx3, j3 = collect_bracketed(L, find(L, r"data3 = \[", i), "[")
    d2 = julia_array(tx2)
    d3 = julia_array(tx3)
    # expansion and mapping to the unit tet as Gridap does it (lines around the tables)
    wx = []
    for w, s, t in d2:
        for x, y, z in ((s, s, t), (s, t, s), (t, s, s), (s, s, s)):
            wx.append([w, x, y, z])
    for w, s, t in d3:
        for x, y, z in ((s, t, t), (t, s, t), (s, s, t), (s, t, s), (t, s, s), (t, t, s)):
            wx.append([w, x, y, z])
    for r in wx:
        r[0] /= 2
        for d in (1, 2, 3):
            r[d] = (r[d] + 1) / 2
    tot = sum(r[0] for r in wx)
    scale = (1 / 6) / tot
    kats["wv_tet_degree4"] = {
        "source": f"{f}:{i + 1}-{j3 + 1}", "npoints": len(wx),
        "points": [r[1:] for r in wx], "weights": [r[0] * scale for r in wx],
        "note": "orbit tables expanded, mapped from [-1,1] to the unit tet, weights scaled "
                "to the tet measure 1/6 (Quadratures.jl _weightcoords_to_coord_weights)"}

    # ---- boundary facets of a 2x2 Cartesian model: order, facet-to-cell map, physical
    # points and normals at the facet points s = 0.25, 0.75 -----------------------------------
    f = "test/GeometryTests/BoundaryTriangulationsTests.jl"
    L = (ref / f).read_text().splitlines()
    i = find(L, r"^model = CartesianDiscreteModel\(domain,partition\)")
    i = find(L, r"^btrian = BoundaryTriangulation\(model\)$", i)
    vals = []
    k = i
    for _ in range(3):
        k = find(L, r"^r = Vector\{Point\{2,Float64\}\}\[", k + 1)
        txt, j = collect_bracketed(L, k, "V")
        vals.append((k, j, julia_array(txt)))
    kats["boundary_facets_2x2"] = {
        "source": f"{f}:{vals[0][0] + 1}-{vals[2][1] + 1}", "domain": [0, 4, 0, 4],
        "partition": [2, 2], "s": [0.25, 0.75], "cell_points": vals[0][2],
        "physical_points": vals[1][2], "normals": vals[2][2]}

    out = HERE / "gridap_kats.json"
    out.write_text(json.dumps(kats, indent=1) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/extract_kats.py <path to a Gridap.jl v0.20.8 checkout>")
    main(pathlib.Path(sys.argv[1]))
