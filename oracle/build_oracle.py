"""Build recipe for the C oracle (test infrastructure, not the product).

``python -m oracle.build_oracle`` compiles ``oracle/tt_oracle.c`` into
``oracle/_build/libtt_oracle.<machine>.so`` with the host gcc.  ``-ffp-contract=off``
keeps multiply-adds unfused so x86_64 and aarch64 hosts give the same bits.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "tt_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtt_oracle.%s.so" % os.uname().machine)


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
