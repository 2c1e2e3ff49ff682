"""Writes reference_kats.json: the known-answer tests of the reference's own test suite.

Each case below is transcribed from the reference's unitTests/tests.cpp (cited by
line). When the reference tree is available (argument or NARVAL_REFERENCE), every case
is verified against the cited line: its `needle` must occur there verbatim, so the
fixture provably carries the reference's numbers. Run:
    python tests/golden/make_reference_kats.py [path/to/reference]
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
INF = "inf"

CASES = [
    # Math.conversionBetweenLCSandWCS (tests.cpp:62-81), precision EPSILON3
    {"test": "Math.conversionBetweenLCSandWCS", "line": 79, "needle": "toLCS(glm::vec3(0, 1, 0), ns, ss, ts), glm::vec3(0, 0, 1)",
     "fn": "to_lcs", "v": [0, 1, 0], "ns": [0, 1, 0], "ss": [1, 0, 0], "ts": [0, 0, 1], "expect": [0, 0, 1], "tol": 1e-3},
    {"test": "Math.conversionBetweenLCSandWCS", "line": 80, "needle": "toWorld(glm::vec3(0, 0, 1), ns, ss, ts), glm::vec3(0, 1, 0)",
     "fn": "to_world", "v": [0, 0, 1], "ns": [0, 1, 0], "ss": [1, 0, 0], "ts": [0, 0, 1], "expect": [0, 1, 0], "tol": 1e-3},
    # Math.generateOrthonormalCS (tests.cpp:86-97): generateOrthonormalCS(normal, v, u)
    {"test": "Math.generateOrthonormalCS", "line": 91, "needle": "vec3EqualsEpsilon(u, glm::vec3(-1, 0, 0)",
     "fn": "orthonormal", "n": [0, 1, 0], "expect_u": [-1, 0, 0], "expect_v": [0, 0, -1], "tol": 1e-3},
    {"test": "Math.generateOrthonormalCS", "line": 96, "needle": "vec3EqualsEpsilon(v, glm::vec3(0, 0, 1)",
     "fn": "orthonormal", "n": [0, -1, 0], "expect_u": [-1, 0, 0], "expect_v": [0, 0, 1], "tol": 1e-3},
]

# Math.sampleUnitSphere (tests.cpp:103-127): sampleUnitSphere(theta / 360, phi / 180)
for line, th, ph, exp in [
    (108, "0.0f", "0.0f", [0, 0, 1]), (109, "90.0f", "0.0f", [0, 0, 1]), (110, "180.0f", "0.0f", [0, 0, 1]),
    (111, "270.0f", "0.0f", [0, 0, 1]), (112, "360.0f", "0.0f", [0, 0, 1]),
    (115, "0.0f", "90.0f", [1, 0, 0]), (116, "90.0f", "90.0f", [0, 1, 0]), (117, "180.0f", "90.0f", [-1, 0, 0]),
    (118, "270.0f", "90.0f", [0, -1, 0]), (119, "360.0f", "90.0f", [1, 0, 0]),
    (122, "0.0f", "180.0f", [0, 0, -1]), (123, "90.0f", "180.0f", [0, 0, -1]), (124, "180.0f", "180.0f", [0, 0, -1]),
    (125, "270.0f", "180.0f", [0, 0, -1]), (126, "360.0f", "180.0f", [0, 0, -1])]:
    e1 = float(th[:-1]) / 360.0
    e2 = float(ph[:-1]) / 180.0
    needle = f"{ph} / 180.0f), glm::vec3({', '.join(str(v) for v in exp)})"
    CASES.append({"test": "Math.sampleUnitSphere", "line": line, "needle": needle, "fn": "sample_unit_sphere",
                  "e1": e1, "e2": e2, "expect": exp, "tol": 1e-3})

# Triangle.intersection (tests.cpp:300-347): vertices (0,0,0), (0,1,0), (1,0,0)
TRI = [[0, 0, 0], [0, 1, 0], [1, 0, 0]]
for line, o, d, hit, point, t in [
    (318, [0, 0, 0], [0, 0, 1], True, [0, 0, 0], 0.0),
    (326, [0, 0, -1], [0, 0, 1], True, [0, 0, 0], 1.0),
    (334, [0, -1, 0], [0, 1, 0], False, None, None),
    (338, [0.25, 0.25, -1], [0, 0, 1], True, [0.25, 0.25, 0], 1.0),
    (345, [0, 0, 1], [0, 0, 1], False, None, None)]:
    fmt = lambda v: ", ".join(("0.25f" if x == 0.25 else str(int(x)) if float(x).is_integer() else str(x)) for x in v)
    CASES.append({"test": "Triangle.intersection", "line": line, "needle": f"ray = {{ glm::vec3({fmt(o)}), glm::vec3({fmt(d)}) }}",
                  "fn": "triangle_intersect", "tri": TRI, "o": o, "d": d, "hit": hit, "point": point, "t": t,
                  "t_exact": True, "tol": 1e-3})

# AABB.intersection (tests.cpp:352-404): box [-0.5, 0.5]^3
for line, o_src, o, hit, point, tn, tf in [
    (372, "0, 0, -1.0", [0, 0, -1.0], True, [0, 0, -0.5], 0.5, 1.5),
    (379, "0, 0, -0.5", [0, 0, -0.5], True, [0, 0, -0.5], 0.0, 1.0),
    (386, "0, -0.5, -0.5", [0, -0.5, -0.5], True, [0, -0.5, -0.5], 0.0, 1.0),
    (393, "0, 0.0, 0.0", [0, 0.0, 0.0], True, [0, 0, -0.5], -0.5, 0.5),
    (400, "0, 0.55, 0.0", [0, 0.55, 0.0], False, None, INF, "-" + INF)]:
    CASES.append({"test": "AABB.intersection", "line": line, "needle": f"ray = {{ glm::vec3({o_src}), glm::vec3(0, 0, 1) }}",
                  "fn": "aabb_intersect", "min": [-0.5, -0.5, -0.5], "max": [0.5, 0.5, 0.5], "o": o, "d": [0, 0, 1],
                  "hit": hit, "point": point, "t_near": tn, "t_far": tf, "tol": 1e-3})

# Model.modelMadeOfTriangles (tests.cpp:409-481)
CUBE = [-0.5, -0.5, -0.5, 0.5, -0.5, -0.5, 0.5, 0.5, -0.5, -0.5, 0.5, -0.5,
        -0.5, -0.5, 0.5, 0.5, -0.5, 0.5, 0.5, 0.5, 0.5, -0.5, 0.5, 0.5]
CUBE_IDX = [0, 1, 3, 1, 2, 3, 5, 1, 2, 2, 5, 6, 4, 5, 6, 6, 4, 7, 4, 0, 3, 3, 7, 4, 7, 6, 2, 2, 3, 7, 4, 5, 1, 1, 0, 4]
for line, needle, o, hit in [(462, "glm::vec3(0, 0, -2), glm::vec3(0, 0, 1)", [0, 0, -2], True),
                             (469, "glm::vec3(1.5, 0, -2), glm::vec3(0, 0, 1)", [1.5, 0, -2], False),
                             (475, "glm::vec3(0, 0, 0), glm::vec3(0, 0, 1)", [0, 0, 0], True)]:
    CASES.append({"test": "Model.modelMadeOfTriangles", "line": line, "needle": needle, "fn": "model_triangles",
                  "verts": CUBE, "indices": CUBE_IDX, "o": o, "d": [0, 0, 1], "t_min": 0.0, "t_max": INF, "hit": hit})
CASES.append({"test": "Model.modelMadeOfTriangles", "line": 419, "needle": "float cube[8 * 3] = { -0.5f, -0.5f, -0.5f,",
              "fn": "none"})
CASES.append({"test": "Model.modelMadeOfTriangles", "line": 429, "needle": "cubeIndices[6 * 2 * 3] = { 0,1,3,",
              "fn": "none"})

# Triangle.area (tests.cpp:683-752)
for line, verts, area in [
    (703, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], 0.5), (711, [[0, 0, 0], [0, 2, 0], [2, 0, 0]], 2.0),
    (719, [[0, 0, 0], [0, 2, 0], [0, 0, 2]], 2.0), (727, [[0, 0, 0], [0, 2, 0], [-2, 0, 0]], 2.0),
    (735, [[0, 0, 0], [0, 2, 0], [0, 0, -2]], 2.0), (743, [[15, 0, 15], [15, 0, 16], [15, 1, 15]], 0.5),
    (751, [[-15, 0, -15], [-15, 0, -16], [-15, -1, -15]], 0.5)]:
    CASES.append({"test": "Triangle.area", "line": line, "needle": "floatEqualsEpsilon(calculatedArea,", "fn": "triangle_area",
                  "tri": verts, "expect": area, "tol": 1e-3})

# Math.isPointInsideTriangleRange (tests.cpp:754-771)
for line, needle, p, exp in [
    (759, "glm::vec3(0.4, 0.4, 0.0)", [0.4, 0.4, 0.0], True), (761, "glm::vec3(0.5, 0.5, 0.0)", [0.5, 0.5, 0.0], True),
    (763, "isPointInsideTriangleRange(v1, v1", [0, 0, 0], True), (764, "isPointInsideTriangleRange(v2, v1", [1, 0, 0], True),
    (765, "isPointInsideTriangleRange(v3, v1", [0, 1, 0], True), (767, "glm::vec3(0.6, 0.6, 0.0)", [0.6, 0.6, 0.0], False),
    (768, "glm::vec3(-0.1, -0.1, 0.0)", [-0.1, -0.1, 0.0], False), (770, "glm::vec3(0.4, 0.4, 0.1)", [0.4, 0.4, 0.1], True)]:
    CASES.append({"test": "Math.isPointInsideTriangleRange", "line": line, "needle": needle, "fn": "point_in_range",
                  "tri": [[0, 0, 0], [1, 0, 0], [0, 1, 0]], "p": p, "expect": exp})

# Triangle.contains (tests.cpp:773-805)
for line, tri, p, exp in [
    (789, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 0, 0], True), (790, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [1, 0, 0], True),
    (791, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 0], True), (792, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0.3, 0.3, 0], True),
    (793, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0.6, 0.6, 0], False), (794, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0.3, 0.3, 0.1], False),
    (795, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [-0.3, -0.3, 0.1], False), (796, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [-0.3, -0.3, 0], False),
    (803, [[0, 0, 0], [1000, 0, 0], [0, 1000, 0]], [0.3, 0.3, 0.1], False),
    (804, [[0, 0, 0], [1000, 0, 0], [0, 1000, 0]], [0.3, 0.3, 0.01], False),
    (805, [[0, 0, 0], [1000, 0, 0], [0, 1000, 0]], [0.3, 0.3, 0.001], False),
    (806, [[0, 0, 0], [1000, 0, 0], [0, 1000, 0]], [0.3, 0.3, 0.0001], False)]:
    def lit(x):
        return str(int(x)) if float(x).is_integer() else str(x)
    CASES.append({"test": "Triangle.contains", "line": line, "needle": "contains(glm::vec3(" + ", ".join(lit(x) for x in p) + "))",
                  "fn": "triangle_contains", "tri": tri, "p": p, "expect": exp})

# Triangle.barycentricCoordinates (tests.cpp:807-839)
for line, p, exp in [(827, [0, 0, 0], [1, 0, 0]), (830, [1, 0, 0], [0, 1, 0]), (833, [0, 1, 0], [0, 0, 1]),
                     (837, [1, 1, 0], [-1, 1, 1])]:
    CASES.append({"test": "Triangle.barycentricCoordinates", "line": line,
                  "needle": "barycentricCoordinates(glm::vec3(" + ", ".join(str(v) for v in p) + ")",
                  "fn": "barycentric", "tri": [[0, 0, 0], [1, 0, 0], [0, 1, 0]], "p": p, "expect": exp, "tol": 1e-3})


def verify(ref_root: str) -> int:
    path = os.path.join(ref_root, "unitTests", "tests.cpp")
    lines = open(path, encoding="latin-1").read().splitlines()
    bad = 0
    for c in CASES:
        text = lines[c["line"] - 1]
        if c["needle"] not in text:
            print(f"line {c['line']} does not contain {c['needle']!r}: {text.strip()!r}")
            bad += 1
    return bad


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NARVAL_REFERENCE", "")
    if ref and os.path.exists(os.path.join(ref, "unitTests", "tests.cpp")):
        bad = verify(ref)
        if bad:
            raise SystemExit(f"{bad} cases do not match the reference test source")
        print(f"verified {len(CASES)} cases against {ref}/unitTests/tests.cpp")
    out = os.path.join(HERE, "reference_kats.json")
    with open(out, "w") as f:
        json.dump({"source": "unitTests/tests.cpp of the reference", "cases": CASES}, f, indent=1)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
