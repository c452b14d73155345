"""Generates xu_translations.json from the reference's known-answer table of
translation coefficients (qpms/tests/testcases_translations_Xu: Xu's
published A and B values at kd = (2, 0.5, 0.5), outgoing Hankel functions,
J. Comput. Phys. 127 (1996) Table II and 139 (1998) Tables 12 and 14), keeping
the entries with n, nu <= 20 as the reference's own test does
(qpms/tests/translations_xutable_test.c:19-25).

Run where the reference tree is: python tests/golden/make_xu_fixture.py
(QPMS_REFERENCE_ROOT overrides /root/reference).
"""
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.environ.get("QPMS_REFERENCE_ROOT", "/root/reference")


def _cx(s):
    # "a + b * I" with C float literals (one entry lacks its exponent letter: ".60669708-10")
    s = s.replace(" ", "").replace("*I", "j").replace("+-", "-")
    s = re.sub(r"(\d)-(\d+)j$", r"\1e-\2j", s)
    return complex(s)


def main():
    txt = open(os.path.join(REF, "qpms", "tests", "testcases_translations_Xu")).read()
    cases = []
    for line in txt.splitlines():
        m = re.match(r"\{QPMS_NORMALISATION_XU,\s*(-?\d+),(-?\d+),(-?\d+),(-?\d+),\s*\{([^}]*)\},\s*"
                     r"QPMS_HANKEL_PLUS,\s*([^,]*),([^}]*)\}", line)
        if not m:
            continue
        mm, n, mu, nu = map(int, m.groups()[:4])
        if n > 20 or nu > 20:
            continue
        kd = [float(x) for x in m.group(5).split(",")]
        A, B = _cx(m.group(6)), _cx(m.group(7))
        cases.append({"m": mm, "n": n, "mu": mu, "nu": nu, "kd": kd, "A": [A.real, A.imag], "B": [B.real, B.imag]})
    with open(os.path.join(ROOT, "tests", "golden", "xu_translations.json"), "w") as f:
        json.dump({"source": "qpms/tests/testcases_translations_Xu (Xu 1996 Table II, 1998 Tables 12, 14)",
                   "J": 3, "cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
