"""Copy the reference's own example inputs used by the tests into this folder.

Caracal ships no expected outputs, but its examples/ inputs are the
fixtures its users run.  The GPU machine has no copy of the reference tree, so
the few files the tests read are committed here, verbatim, by this script:

  calc_rate/h+h2/       rate.key, ts.xyz          (H + H2 rate at 300 K)
  dynamic/glutathione/  glutathione.key, .qmdff, start.xyz
  evbopt/dE-EVB/        evbopt.key, min1/min2.qmdff, ref.dat, struc.xyz
  explore/ts_irc_ch4oh/ ts.key, irc.key, ts_start.xyz (CH4 + OH saddle and IRC)

Run: python tests/golden/reference/copy_inputs.py [path of the Caracal tree]
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = {
    "calc_rate/h+h2": ["rate.key", "ts.xyz"],
    "dynamic/glutathione": ["glutathione.key", "glutathione.qmdff", "start.xyz"],
    "evbopt/dE-EVB": ["evbopt.key", "min1.qmdff", "min2.qmdff", "ref.dat", "struc.xyz"],
    "explore/ts_irc_ch4oh": ["ts.key", "irc.key", "ts_start.xyz"],
}


def main(tree="/root/reference"):
    for sub, names in FILES.items():
        dst = os.path.join(HERE, sub)
        os.makedirs(dst, exist_ok=True)
        for n in names:
            shutil.copyfile(os.path.join(tree, "examples", sub, n), os.path.join(dst, n))
            print(os.path.join(sub, n))


if __name__ == "__main__":
    main(*sys.argv[1:])
