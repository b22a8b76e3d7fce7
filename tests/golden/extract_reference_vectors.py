"""Extracts the golden vectors of the reference's own test suite into JSON.

Reads the Boost.Compute test sources (``test/test_*.cpp`` under the reference
checkout given by ``--reference``) as text, pulls the literal input arrays and
the literal expected values out of each listed test case, and writes
``reference_vectors.json`` next to this script.  Nothing is executed: the
reference needs OpenCL and Boost, neither of which is installed here, so its own
known-answer tests are the pin for the oracle and the CUDA path.

Every case records its source file and line range so it can be checked
against the reference by hand.  Run:

    python tests/golden/extract_reference_vectors.py --reference <checkout>
"""
from __future__ import annotations

import argparse
import json
import re
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "reference_vectors.json"

# ---------------------------------------------------------------------------
# Case table: which test case, which lines, what operation it pins, and which
# literal arrays in those lines are its input and expected output.
#   input: name of a `T name[] = {...}` array (or list of names)
#   expect: (target variable of CHECK_RANGE_EQUAL, occurrence index)
#   scalars: (op, init) per BOOST_CHECK_EQUAL in order, for reduce/accumulate
R = "test/test_radix_sort.cpp"
RK = "test/test_radix_sort_by_key.cpp"
S = "test/test_sort.cpp"
SK = "test/test_sort_by_key.cpp"
SSK = "test/test_stable_sort_by_key.cpp"
INS = "test/test_insertion_sort.cpp"
SC = "test/test_scan.cpp"
RD = "test/test_reduce.cpp"
AC = "test/test_accumulate.cpp"
RBK = "test/test_reduce_by_key.cpp"
TF = "test/test_transform.cpp"

TYPES = ["char", "uchar", "short", "ushort", "int", "uint", "long", "ulong", "float", "double"]
RADIX_ASC = [(29, 49), (51, 67), (69, 85), (87, 103), (105, 119), (121, 137), (139, 155),
             (157, 173), (175, 202), (204, 227)]
RADIX_DESC = [(229, 255), (257, 283), (285, 311), (313, 339), (341, 367), (369, 395), (397, 423),
              (425, 451), (453, 494), (496, 528)]
SORT_TYPED = [(79, 91), (93, 105), (107, 119), (121, 133), (135, 145), (147, 159), (161, 173),
              (175, 187), (189, 203), (205, 225)]
INS_TYPED = [(24, 36), (38, 50), (52, 64), (66, 78), (80, 90), (92, 104), (106, 118), (120, 132),
             (134, 148), (150, 171)]

CASES: list[dict] = []
for t, (a, b) in zip(TYPES, RADIX_ASC):
    CASES.append(dict(id=f"radix_sort_{t}", file=R, lines=[a, b], kind="radix_sort", dtype=t,
                      descending=False, input="data", expect=("vector", -1)))
for t, (a, b) in zip(TYPES, RADIX_DESC):
    CASES.append(dict(id=f"radix_sort_{t}_desc", file=R, lines=[a, b], kind="radix_sort", dtype=t,
                      descending=True, input="data", expect=("vector", -1)))
CASES.append(dict(id="radix_sort_partial_vector", file=R, lines=[530, 543], kind="radix_sort_range",
                  dtype="int", descending=False, input="data", range=[2, 8], expect=("vec", -1)))
for name, (a, b), kt, vt, desc in [
        ("int_by_int", (30, 61), "int", "int", False), ("int_by_int_desc", (63, 100), "int", "int", True),
        ("uint_by_uint", (102, 129), "uint", "uint", False),
        ("uint_by_uint_desc", (131, 169), "uint", "uint", True),
        ("int_by_float", (171, 198), "float", "int", False),
        ("int_by_float_desc", (200, 238), "float", "int", True),
        ("char_by_int", (240, 265), "int", "char", False), ("int2_by_int", (267, 311), "int", "int2", False)]:
    CASES.append(dict(id=f"radix_sort_by_key_{name}", file=RK, lines=[a, b], kind="radix_sort_by_key",
                      dtype=kt, value_dtype=vt, descending=desc, input=["keys_data", "values_data"],
                      expect=[("keys", -1), ("values", -1)]))
for t, (a, b) in zip(TYPES, SORT_TYPED):
    CASES.append(dict(id=f"sort_{t}", file=S, lines=[a, b], kind="sort", dtype=t, descending=False,
                      input="data", expect=("vector", -1)))
CASES.append(dict(id="sort_float_3", file=S, lines=[71, 77], kind="sort", dtype="float", descending=False,
                  input="data", expect=("vec", -1)))
CASES.append(dict(id="sort_reverse_int", file=S, lines=[227, 236], kind="sort", dtype="int", descending=True,
                  input="data", expect=("vector", -1)))
CASES.append(dict(id="sort_host_vector", file=S, lines=[286, 292], kind="sort", dtype="int", descending=False,
                  input="data", expect=("vector", -1)))
for t, (a, b) in zip(TYPES, INS_TYPED):
    CASES.append(dict(id=f"insertion_sort_{t}", file=INS, lines=[a, b], kind="insertion_sort", dtype=t,
                      descending=False, input="data", expect=("vector", -1)))
CASES.append(dict(id="sort_by_key_char_by_int", file=SK, lines=[79, 91], kind="sort_by_key", dtype="int",
                  value_dtype="char", descending=False, input=["keys_data", "values_data"],
                  expect=[("keys", -1), ("values", -1)]))
for name, (a, b), kt, vt in [("int_by_int", (73, 95), "int", "int"), ("uint_by_uint", (97, 119), "uint", "uint"),
                             ("int_by_float", (121, 143), "float", "int"), ("char_by_int", (145, 163), "int", "char")]:
    CASES.append(dict(id=f"stable_sort_by_key_{name}", file=SSK, lines=[a, b], kind="sort_by_key", dtype=kt,
                      value_dtype=vt, descending=False, input=["keys_data", "values_data"],
                      expect=[("keys", -1), ("values", -1)]))
# scans
CASES += [
    dict(id="inclusive_scan_int", file=SC, lines=[41, 60], kind="scan", dtype="int", op="plus", exclusive=False,
         input="data", expect=("result", 0)),
    dict(id="exclusive_scan_int", file=SC, lines=[91, 110], kind="scan", dtype="int", op="plus", exclusive=True,
         init=0, input="data", expect=("result", 0)),
    dict(id="inclusive_scan_doctest", file=SC, lines=[287, 306], kind="scan", dtype="int", op="plus",
         exclusive=False, input="data", expect=("output", -1)),
    dict(id="exclusive_scan_doctest", file=SC, lines=[308, 327], kind="scan", dtype="int", op="plus",
         exclusive=True, init=0, input="data", expect=("output", -1)),
    dict(id="inclusive_scan_int_multiplies", file=SC, lines=[329, 358], kind="scan", dtype="int",
         op="multiplies", exclusive=False, input="data", expect=("output", 0)),
    dict(id="exclusive_scan_int_multiplies", file=SC, lines=[360, 390], kind="scan", dtype="int",
         op="multiplies", exclusive=True, init=10, input="data", expect=("output", 0)),
]
# reductions: (op, init) for each BOOST_CHECK_EQUAL in order; init None = reduce
CASES += [
    dict(id="reduce_int", file=RD, lines=[29, 40], kind="fold", dtype="int", input="data",
         scalars=[("plus", None), ("multiplies", None)]),
    dict(id="reduce_doctest", file=RD, lines=[51, 62], kind="fold", dtype="int", input="data",
         scalars=[("plus", None)]),
    dict(id="reduce_int_min_max", file=RD, lines=[90, 113], kind="fold", dtype="int", input="data",
         scalars=[("min", None), ("max", None)]),
    dict(id="reduce_pinned_vector", file=RD, lines=[137, 155], kind="fold", dtype="int", input="data",
         scalars=[("plus", None)]),
    dict(id="accumulate_sum_int", file=AC, lines=[25, 43], kind="fold", dtype="int", input="data",
         scalars=[("plus", 0), ("plus", -10), ("plus", 5)]),
    dict(id="accumulate_product_int", file=AC, lines=[45, 69], kind="fold", dtype="int", input="data",
         scalars=[("multiplies", 1), ("multiplies", -1), ("multiplies", 2)]),
    dict(id="accumulate_quotient_int", file=AC, lines=[71, 85], kind="fold", dtype="int", input="data",
         scalars=[("divides", 1024)]),
    dict(id="accumulate_min_max_float", file=AC, lines=[227, 257], kind="fold", dtype="float", input="data",
         scalars=[("min", "FLT_MAX"), ("max", "FLT_MIN"), ("min", -1.0), ("max", 10.0)]),
]
# generated-input reductions whose inputs the test builds with iota/fill
CASES += [
    dict(id="accumulate_sum_iota", file=AC, lines=[150, 206], kind="fold_iota", dtype="int",
         sizes=[0, 0, 50, 50, 1000, 1000, 1025, 1025], scalars=[("plus", 0), ("plus", 4), ("plus", 0),
                                                                  ("plus", 11), ("plus", 0), ("plus", -45),
                                                                  ("plus", 0), ("plus", 2)]),
]
CASES += [
    dict(id="reduce_by_key_int", file=RBK, lines=[26, 46], kind="reduce_by_key", dtype="int", value_dtype="int",
         op="plus", input=["keys", "data"], expect=[("keys_output", -1), ("values_output", -1)]),
    dict(id="reduce_by_key_int_one_key_value", file=RBK, lines=[90, 106], kind="reduce_by_key", dtype="int",
         value_dtype="int", op="plus", input=["keys", "data"], expect=[("keys_output", -1), ("values_output", -1)]),
    dict(id="reduce_by_key_int_min", file=RBK, lines=[108, 125], kind="reduce_by_key", dtype="int",
         value_dtype="int", op="min", input=["keys", "data"], expect=[("keys_output", 0), ("values_output", 0)]),
    dict(id="reduce_by_key_int_max", file=RBK, lines=[108, 132], kind="reduce_by_key", dtype="int",
         value_dtype="int", op="max", input=["keys", "data"], expect=[("keys_output", 1), ("values_output", 1)]),
    dict(id="transform_int_abs", file=TF, lines=[29, 41], kind="transform_unary", dtype="int", op="abs",
         input="data", expect=("vector", -1)),
    dict(id="transform_abs_doctest", file=TF, lines=[282, 299], kind="transform_unary", dtype="int", op="abs",
         input="data", expect=("vec", -1)),
    dict(id="transform_add_int", file=TF, lines=[75, 91], kind="transform_binary", dtype="int", op="plus",
         input=["data1", "data2"], expect=("output", 0)),
    dict(id="transform_multiplies_int", file=TF, lines=[75, 99], kind="transform_binary", dtype="int",
         op="multiplies", input=["data1", "data2"], expect=("output", 1)),
]

# ---------------------------------------------------------------------------
_CHAR_ESC = {"0": 0, "n": 10, "t": 9, "\\": 92, "'": 39}


def _number(tok: str):
    tok = tok.strip()
    m = re.fullmatch(r"(?:compute::|boost::compute::|bc::)?int2_\(\s*([^,]+),\s*([^)]+)\)", tok)
    if m:
        return [_number(m.group(1)), _number(m.group(2))]
    if tok.startswith("'"):
        body = tok[1:-1]
        if body.startswith("\\"):
            return _CHAR_ESC[body[1:]]
        return ord(body)
    if re.fullmatch(r"-?0[xX][0-9a-fA-F]+", tok):
        return int(tok, 16)
    if re.fullmatch(r"-?\d+", tok):
        return int(tok)
    t = tok.rstrip("fF")
    return float(t)


def _split_top(s: str) -> list[str]:
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [c.strip() for c in out if c.strip()]


def _balanced(text: str, start: int) -> tuple[str, int]:
    """text[start] == '('; returns the inside and the index after ')'."""
    depth = 0
    for i in range(start, len(text)):
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:i], i + 1
    raise ValueError("unbalanced parentheses")


def _strip_comments(text: str) -> str:
    return re.sub(r"//[^\n]*", "", text)


def parse_block(text: str) -> dict:
    text = _strip_comments(text)
    arrays = {}
    for m in re.finditer(r"(\w+)\s*\[\s*\]\s*=\s*\{(.*?)\}\s*;", text, re.S):
        arrays[m.group(1)] = [_number(t) for t in _split_top(m.group(2))]
    checks: dict[str, list] = {}
    for m in re.finditer(r"CHECK_RANGE_EQUAL\s*\(", text):
        inner, _ = _balanced(text, m.end() - 1)
        parts = _split_top(inner)
        var, lst = parts[2], parts[3].strip()
        assert lst.startswith("(") and lst.endswith(")"), lst
        checks.setdefault(var, []).append([_number(t) for t in _split_top(lst[1:-1])])
    scalars = []
    for m in re.finditer(r"BOOST_CHECK_EQUAL\s*\(", text):
        inner, _ = _balanced(text, m.end() - 1)
        parts = _split_top(inner)
        last = parts[-1]
        try:
            scalars.append(_number(last))
        except (ValueError, KeyError):
            pass
    return {"arrays": arrays, "checks": checks, "scalars": scalars}


def extract(reference: Path) -> list[dict]:
    out = []
    for c in CASES:
        lines = (reference / c["file"]).read_text().splitlines()
        a, b = c["lines"]
        block = parse_block("\n".join(lines[a - 1:b]))
        case = {k: v for k, v in c.items() if k not in ("input", "expect", "scalars")}
        if "input" in c:
            names = c["input"] if isinstance(c["input"], list) else [c["input"]]
            case["inputs"] = [block["arrays"][nm] for nm in names]
        if "expect" in c:
            exps = c["expect"] if isinstance(c["expect"], list) else [c["expect"]]
            case["expected"] = [block["checks"][var][idx] for var, idx in exps]
        if "scalars" in c:
            vals = [v for v in block["scalars"] if not isinstance(v, list)]
            if c["kind"] == "fold":
                # drop size checks that precede the value checks
                vals = vals[-len(c["scalars"]):]
            assert len(vals) >= len(c["scalars"]), (c["id"], vals)
            vals = vals[-len(c["scalars"]):]
            case["checks"] = [{"op": op, "init": init, "expected": v} for (op, init), v in zip(c["scalars"], vals)]
        out.append(case)
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, type=Path)
    args = ap.parse_args()
    cases = extract(args.reference)
    OUT.write_text(json.dumps({"source": "boostorg/compute test suite (test/test_*.cpp)",
                               "generator": "tests/golden/extract_reference_vectors.py",
                               "cases": cases}, indent=1) + "\n")
    print(f"wrote {len(cases)} cases to {OUT}")


if __name__ == "__main__":
    main()
