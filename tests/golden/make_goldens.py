"""Extracts the reference's golden values into tests/golden/test_ci.json.

The reference package's own test suite (tests/testthat/test-ci.R of
EDM-Developers/fastEDM-r) pins the prediction path with literal rho values
and with Stata-generated random vectors used as inputs.  This script reads
that file as text (it never runs R) and records:

  vectors: the inline input vectors, keyed by test block and name;
  lines:   for every line holding expected values (check_edm_result(s),
           check_noisy_edm_result, expect_approx_equal, `rho... <- c(...)`),
           the numeric literals on that line, keyed by 1-based line number.

Run it where the reference checkout is available:
    python tests/golden/make_goldens.py /path/to/fastEDM-r
"""
import json
import re
import sys
from pathlib import Path

NUM = r"-?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"

VECTOR_LINES = {
    # test block "Simple manifolds": normal rv's from Stata, seed 12345678
    "simple_u1": 89,
    # test block "Missing data manifolds": uniform rv's, seed 12345678
    "missing_u": 227,
    # test block "From 'bigger-test.do' script"
    "bigger_u": 301,
    "bigger_u1": 304,
}

EXPECT_PAT = re.compile(
    r"check_edm_results?\(|check_noisy_edm_result\(|expect_approx_equal\(|"
    r"^\s*(?:co_)?rho[0-9_a-z]*\s*<-\s*c\(|absErr"
)


def numbers_in(text):
    """Numeric literals in order; R's NA becomes None."""
    return [None if v == "NA" else float(v) for v in re.findall(NUM + r"|\bNA\b", text)]


def main(ref_root):
    src = Path(ref_root) / "tests" / "testthat" / "test-ci.R"
    lines = src.read_text().splitlines()
    out = {"source": "tests/testthat/test-ci.R", "vectors": {}, "lines": {}}
    for name, ln in VECTOR_LINES.items():
        text = lines[ln - 1]
        body = text[text.index("c(") + 2 : text.rindex(")")]
        out["vectors"][name] = numbers_in(body)
    for i, text in enumerate(lines, start=1):
        if EXPECT_PAT.search(text):
            # drop identifiers like res1/rho2/E so only literal values remain
            cleaned = re.sub(r"\b(?!NA\b)[A-Za-z_][A-Za-z_0-9.]*", " ", text)
            vals = numbers_in(cleaned)
            out["lines"][str(i)] = {"text": text.strip(), "values": vals}
    dst = Path(__file__).with_name("test_ci.json")
    dst.write_text(json.dumps(out, indent=1))
    print(f"wrote {dst}: {len(out['vectors'])} vectors, {len(out['lines'])} expectation lines")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_goldens.py /path/to/fastEDM-r")
    main(sys.argv[1])
