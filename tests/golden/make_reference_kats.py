"""Extract the known-answer values of the reference's own test suite into reference_kats.json.

The reference (HDiscontinuousGalerkin.jl) is Julia and cannot run in this environment, so
its golden numbers are read from its test files as text and evaluated here.  Run this only
where the reference tree is present; the resulting JSON is committed and is what the tests
read.  Usage:  python tests/golden/make_reference_kats.py /path/to/reference
"""
import json
import math
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HDG_REFERENCE_TREE", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")

_ENV = {"sqrt": math.sqrt, "sq2": math.sqrt(2.0), "sq3": math.sqrt(3.0), "pi": math.pi, "π": math.pi}


def _eval(expr: str) -> float:
    """Value of an arithmetic expression read from the reference's test files.  The text is parsed,
    never executed: only numbers, the names in _ENV, + - * / ** (Julia's ^ and //), unary signs and
    calls of sqrt are accepted; anything else raises ValueError."""
    import ast
    import operator
    expr = expr.replace("^", "**").replace("//", "/")
    binops = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
              ast.Pow: operator.pow}
    unops = {ast.UAdd: operator.pos, ast.USub: operator.neg}

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)) and not isinstance(node.value, bool):
            return float(node.value)
        if isinstance(node, ast.Name) and node.id in _ENV and node.id != "sqrt":
            return float(_ENV[node.id])
        if isinstance(node, ast.BinOp) and type(node.op) in binops:
            return binops[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.UnaryOp) and type(node.op) in unops:
            return unops[type(node.op)](ev(node.operand))
        if (isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id == "sqrt"
                and len(node.args) == 1 and not node.keywords):
            return math.sqrt(ev(node.args[0]))
        raise ValueError(f"not a plain arithmetic expression: {expr!r}")
    return ev(ast.parse(expr, mode="eval"))


def julia_matrix(text: str):
    """Evaluate a Julia matrix literal such as `-[a b; c d]` (space-separated elements)."""
    text = text.strip()
    neg = text.startswith("-")
    body = text[text.index("[") + 1: text.rindex("]")]
    rows = [r for r in (x.strip() for x in body.replace("\n", " ").split(";")) if r]
    mat = [[_eval(e) for e in r.split()] for r in rows]
    if neg:
        mat = [[-v for v in r] for r in mat]
    return mat


def grab_assignments(src: str, name: str):
    """All `name[k] = <matrix literal>` assignments (a literal may span lines)."""
    out = {}
    for m in re.finditer(re.escape(name) + r"\[(\d)\]\s*=\s*(-?\[)", src):
        k = int(m.group(1))
        start = m.start(2)
        depth, i = 0, src.index("[", start)
        while True:
            if src[i] == "[":
                depth += 1
            elif src[i] == "]":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        out[k] = julia_matrix(src[start: i + 1])
    for m in re.finditer(re.escape(name) + r"\[(\d)\]\s*=\s*" + re.escape(name) + r"\[(\d)\]", src):
        out[int(m.group(1))] = out[int(m.group(2))]
    return [out[k] for k in sorted(out)]


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("pass the reference tree as the first argument")
    t = lambda p: open(os.path.join(REF, p)).read()
    fs = t("test/test_FunctionSpace.jl")
    sfs = t("test/test_ScalarFuncSp.jl")
    mesh = t("test/test_mesh.jl")
    quad = t("test/test_quadrature.jl")
    hand = t("test/test_handlers.jl")
    ex = t("examples/poisson2D_HDG.jl")

    kats = {"source": "HDiscontinuousGalerkin.jl test suite (values evaluated from its test files)"}
    # test/test_FunctionSpace.jl:49-72 golden element blocks on test/mesh/figure2.1, p=1, tau=1
    kats["figure2_1_Be"] = grab_assignments(fs, "Be_ex")
    kats["figure2_1_Ce"] = grab_assignments(fs, "Ce_ex")
    kats["figure2_1_Ee"] = grab_assignments(fs, "Ee_ex")
    kats["figure2_1_He"] = grab_assignments(fs, "He_ex")
    # :39-41 face detJdS of the last reinit!-ed cell
    kats["figure2_1_facedetJdS_last_cell"] = [_eval(m.group(1)) for m in
                                              re.finditer(r"getfacedetJdS\(Mh, \d, 1\) ≈ (\S+)", fs)]
    kats["figure2_1_Ae_scale"] = _eval(re.search(r"@test Ae ≈ (\S+)\*one\(Ae\)", fs).group(1))
    kats["figure2_1_local_dofs"] = [int(m.group(1)) for m in re.finditer(r"getnlocaldofs\(\w+\) == (\d+)", fs)]
    kats["figure2_1_errornorm_sq_max"] = _eval(re.search(r"@test Etu_h <= (\S+)", fs).group(1))
    # examples/poisson2D_HDG.jl:37,217-218: 10x10 mesh bound
    kats["rect10_errornorm_sq_max"] = _eval(re.search(r"Etu_h <= (\S+)", ex).group(1))
    # test/test_ScalarFuncSp.jl:15-33 geometry
    kats["figure2_1_Jinv"] = [julia_matrix(m.group(1)) for m in re.finditer(r"Tensor\{2,2\}\((\[[^\]]*\])\)", sfs)]
    dj = re.search(r"detsJf = \((.*?)\)\n@test", sfs, re.S).group(1)
    kats["figure2_1_detJf"] = [[_eval(e) for e in r.split(",")] for r in re.findall(r"\[([^\]]*)\]", dj)]
    kats["figure2_1_detJ"] = _eval(re.search(r"Wh\.detJ\[\] ≈ (\S+)", sfs).group(1))
    nr = re.search(r"Wh\.normals ≈ \[(.*)\]\n", sfs).group(1)
    kats["figure2_1_cell1_normals"] = [[_eval(e) for e in v.split(",")] for v in re.findall(r"Vec\{2\}\(\[([^\]]*)\]\)", nr)]
    # test/test_mesh.jl:11-44 numbering
    mats = re.findall(r"getcells_matrix\(mesh\) == (\[[^\]]*\])", mesh)
    verts = re.findall(r"get_vertices_matrix\(mesh\) == (\[[^\]]*\])", mesh)
    kats["figure2_1_cells"] = [[int(v) for v in r] for r in julia_matrix(mats[0])]
    kats["figure2_1_vertices"] = julia_matrix(verts[0])
    kats["rect2x2_cells"] = [[int(v) for v in r] for r in julia_matrix(mats[1])]
    kats["rect2x2_vertices"] = julia_matrix(verts[1])
    cf = re.findall(r"mesh\.cells\[1\]\.faces == \(([^)]*)\)", mesh)
    kats["figure2_1_cell1_faces"] = [int(v) for v in cf[0].split(",")]
    kats["rect2x2_cell1_faces"] = [int(v) for v in cf[1].split(",")]
    orr = re.findall(r"face_orientation\(mesh,1,i\) for i in 1:3\] == \[([^\]]*)\]", mesh)
    kats["figure2_1_cell1_orientation"] = [v.strip() == "true" for v in orr[0].split(",")]
    kats["rect2x2_cell1_orientation"] = [v.strip() == "true" for v in orr[1].split(",")]
    bs = re.findall(r'getfaceset\(mesh, "boundary"\) == Set\(\[([^\]]*)\]\)', mesh)
    kats["figure2_1_boundary"] = sorted(int(v) for v in bs[0].split(","))
    kats["rect2x2_boundary"] = sorted(int(v) for v in bs[1].split(","))
    cd = re.findall(r"cell_diameter\(mesh,1\) == (\S+)", mesh)
    kats["figure2_1_cell1_diameter"] = _eval(cd[0])
    kats["rect2x2_cell1_diameter"] = _eval(cd[1])
    kats["figure2_1_cell_volume"] = _eval(re.findall(r"≈ (1/\d)", mesh)[0])
    kats["rect2x2_cell_volume"] = _eval(re.findall(r"≈ (1/\d)", mesh)[1])
    # test/test_quadrature.jl:6-25
    gm1 = re.search(r"getweights\(quad_rule\) ≈ 0\.5\*\[([^\]]*)\]", quad).group(1)
    kats["gm1_weights"] = [0.5 * _eval(v) for v in gm1.split(",")]
    kats["gm1_points"] = [[_eval(e) for e in m.group(1).split(",")] for m in
                          re.finditer(r"getpoints\(quad_rule\)\[\d\] ≈ \[([^\]]*)\]", quad)][1:]
    kats["gm0_points"] = [[_eval(e) for e in m.group(1).split(",")] for m in
                          re.finditer(r"getpoints\(quad_rule\)\[\d\] ≈ \[([^\]]*)\]", quad)][:1]
    # test/test_handlers.jl:13-21 DofHandler on the 2x2 mesh, P1
    kats["rect2x2_p1_cell_dofs"] = [int(v) for v in re.search(r"dh\.cell_dofs == \[([^\]]*)\]", hand).group(1).split(",")]
    kats["rect2x2_p1_cell_dofs_offset"] = [int(v) for v in
                                           re.search(r"dh\.cell_dofs_offset == \[([^\]]*)\]", hand).group(1).split(",")]
    kats["rect2x2_p1_prescribed"] = [int(v) for v in
                                     re.search(r"dbc\.prescribed_dofs == \[([^\]]*)\]", hand).group(1).split(",")]
    with open(OUT, "w") as fh:
        json.dump(kats, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
