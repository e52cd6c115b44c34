"""Extract the element data Caracal's QMDFF set-up uses into qmdff_tables.npz.

QMDFF's non-bonded terms need Grimme's D3 data as Caracal carries it: the
C6 reference table (src/copyc6.f90, 32385 lines of C6, element/CN-index
codes and the two reference coordination numbers), the D3 cut-off radii
(src/setr0.f90, 4465 values), r2r4 and the covalent radii rcov of the CN
(src/setnonb.f90:53-102) and the covalent radii rad (src/prepare.f90:177-191).
These are tables the force field is defined by, so they are taken over as
data, value by value.  Literals without a D exponent are REAL(4) in the
reference (no -fdefault-real-8 in its Makefile) and are stored here rounded
to float32 as gfortran widens them; D-exponent literals are stored as the
nearest double.

Run: python caracal_gb300/data/make_qmdff_tables.py [path of the Caracal tree]
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = re.compile(r"[-+]?\d+\.\d*(?:[DdEe][-+]?\d+)?")


def _strip(line):
    i = line.find("!")
    return line if i < 0 else line[:i]


def constructor_values(text, name):
    """All numeric literals of the array constructors assigned to `name`
    (`name(a:b)=(/ ... /)` or `name = (/ ... /)`), in order, as
    (string, is_double) pairs."""
    out = []
    lines = text.splitlines()
    i = 0
    head = re.compile(r"^\s*" + re.escape(name) + r"\s*(\([^)]*\))?\s*=\s*\(/", re.I)
    while i < len(lines):
        if head.match(_strip(lines[i])):
            body = _strip(lines[i]).split("(/", 1)[1]
            while "/)" not in body:
                i += 1
                body += " " + _strip(lines[i])
            body = body.split("/)", 1)[0]
            for tok in NUM.findall(body.replace("&", " ")):
                out.append((tok, "d" in tok.lower()))
        i += 1
    return out


def to_array(vals):
    a = np.zeros(len(vals))
    for k, (tok, dbl) in enumerate(vals):
        x = float(tok.replace("D", "E").replace("d", "e"))
        a[k] = x if dbl else float(np.float32(x))
    return a


def main(tree="/root/reference"):
    src = os.path.join(tree, "src")
    read = lambda n: open(os.path.join(src, n)).read()  # noqa: E731
    pars = to_array(constructor_values(read("copyc6.f90"), "pars"))
    assert pars.size == 161925, pars.size
    r0ab = to_array(constructor_values(read("setr0.f90"), "r0ab"))
    assert r0ab.size == 4465, r0ab.size
    setnonb = read("setnonb.f90")
    r2r4 = to_array(constructor_values(setnonb, "r2r4"))
    rcov = to_array(constructor_values(setnonb, "rcov"))
    rad = to_array(constructor_values(read("prepare.f90"), "rad"))
    assert r2r4.size == rcov.size == rad.size == 94
    np.savez_compressed(os.path.join(HERE, "qmdff_tables.npz"), d3_pars=pars.reshape(-1, 5), r0ab_ref=r0ab,
                        r2r4=r2r4, rcov=rcov, rad_angstrom=rad)
    print("d3_pars", pars.reshape(-1, 5).shape, "r0ab", r0ab.shape, "r2r4/rcov/rad", r2r4.shape)


if __name__ == "__main__":
    main(*sys.argv[1:])
