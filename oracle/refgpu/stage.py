#!/usr/bin/env python3
"""Stages the reference's modeling programs for a build on the GPU machine.

TEST INFRASTRUCTURE.  The reference's stepping path runs only on a GPU through
cuFFT, and the GPU machine has no copy of the reference tree, so this script
(run where the reference tree is mounted) copies the files of its two modeling
programs (sgpstd-qmodeling: the aps and vaps mains, acps4.cu, acsglw.cu,
funca.c, func.c, src.c and their headers) to baseline/_ref/src, which git
ignores and which travels with the working tree.  It writes one more pair of
files there: the two mains with `#define pml 10` changed to 20 (the CPML width
of the aps and vaps workloads).  oracle/refgpu/Makefile builds them.

    python oracle/refgpu/stage.py [reference tree]   # default: $QPSTD_REFERENCE,
                                                      # else ../reference beside the repo
"""
import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
FILES = ["acousticsgps4.c", "visacousticsgps4.c", "acps4.cu", "acsglw.cu", "funca.c", "func.c", "src.c",
         "statement.h", "revolve.h"]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else (os.environ.get("QPSTD_REFERENCE")
                                                 or os.path.join(os.path.dirname(ROOT), "reference"))
    src = os.path.join(ref, "sgpstd-qmodeling")
    if not os.path.isdir(src):
        raise SystemExit(f"no reference tree at {ref}")
    dst = os.path.join(ROOT, "baseline", "_ref", "src")
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        os.chmod(os.path.join(dst, f), 0o644)
    for main in ("acousticsgps4.c", "visacousticsgps4.c"):
        txt = open(os.path.join(src, main)).read()
        if "#define pml 10" not in txt:
            raise SystemExit(f"{main}: the CPML width is not the expected '#define pml 10'")
        out = os.path.join(dst, main.replace(".c", "_pml20.c"))
        open(out, "w").write(txt.replace("#define pml 10", "#define pml 20", 1))
    print(f"staged {len(FILES)} files (+2 patched mains) into {dst}")


if __name__ == "__main__":
    main()
