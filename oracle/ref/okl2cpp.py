"""Translate the reference's BS OKL kernels for OCCA Serial execution (checker only).

OCCA's Serial backend runs an OKL kernel as plain nested loops: every @outer and
@inner loop (and @tile) becomes an ordinary for loop, consecutive @inner loops run
one after the other (the implicit barrier), @shared arrays become locals and
@restrict becomes __restrict__.  This does the same textual lowering for the
subset of OKL the BS1-BS5 kernels use, writing C++ to stdout.  Usage:
    python okl2cpp.py <file.okl> <suffix>
Kernel names get `suffix` appended so one object can hold several block sizes.
"""
import re
import sys


def lower(src: str, suffix: str) -> str:
    src = re.sub(r"@kernel\s+void\s+(\w+)", lambda m: f'extern "C" void {m.group(1)}{suffix}', src)
    # OKL puts @restrict before the pointee type; C++ wants it after the '*'
    src = re.sub(r"@restrict\s+([^,()]*?)\*\s*(\w+)", r"\1* __restrict__ \2", src)
    src = src.replace("@shared", "").replace("@exclusive", "")
    src = re.sub(r";\s*@tile\([^)]*\)\s*\)", ")", src)
    src = re.sub(r";\s*@(outer|inner)(\(\d\))?\s*\)", ")", src)
    if "@" in re.sub(r"//.*", "", src):
        raise SystemExit("unsupported OKL construct left after lowering")
    return src


if __name__ == "__main__":
    text = open(sys.argv[1]).read()
    sys.stdout.write(lower(text, sys.argv[2] if len(sys.argv) > 2 else ""))
