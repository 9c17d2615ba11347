"""covcount-compatible command line on the GPU finisher.

Drop-in for the finisher binary covengine runs after a search
(BIN['covcount'], cov/engine/covengine:71, :727-753): same flags (-q -n -R
-M --in [--out] [--fast], cov/engine/covcount.c:66-85), same
`COUNT q= n= R= M= words= uncovered=` line, same --out file (M distinct
base-36 words, written to <out>.part and renamed) and exit status (0 iff
covered, 1 otherwise and always with --fast, 2 on bad arguments).
"""
import sys

from . import codefile, verify
from .lib import CovError


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    q = n = M = 0
    R = -1
    inp = outp = None
    fast = False
    i = 0
    while i < len(argv):
        a = argv[i]
        if a in ("-q", "-n", "-R", "-M", "--in", "--out") and i + 1 < len(argv):
            v = argv[i + 1]
            i += 2
            if a == "-q": q = int(v)
            elif a == "-n": n = int(v)
            elif a == "-R": R = int(v)
            elif a == "-M": M = int(v)
            elif a == "--in": inp = v
            else: outp = v
            continue
        if a == "--fast":
            fast = True
            i += 1
            continue
        sys.stderr.write("bad option %s\n" % a)
        return 2
    if q < 2 or n < 1 or R < 0 or M < 1 or not inp:
        sys.stderr.write("usage: covcount -q Q -n N -R R -M M --in f [--out g]\n")
        return 2
    code = codefile.read_code_finisher(inp, q, n, M)
    try:
        out, unc = verify.finish(code, q, n, R, M, fast=fast)
    except CovError as e:
        sys.stderr.write("covcount_gpu: %s\n" % e)
        return 2
    print("COUNT q=%d n=%d R=%d M=%d words=%d uncovered=%d" % (q, n, R, M, len(out), unc))
    sys.stdout.flush()
    if outp:
        body = codefile.format_code(out, q)
        tmp = outp + ".part"
        with open(tmp, "w") as f:
            f.write(body)
        import os
        os.replace(tmp, outp)
    if fast:
        return 1
    return 0 if unc == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
