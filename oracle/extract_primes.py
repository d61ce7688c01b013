"""Writes oracle/permutation_primes.inc, the prime table of the reference's
PermutationMapper (BEPUutilities/PermutationMapper.cs:49-104).

The table is data the reference-order mode must reproduce exactly, so it is
extracted from the reference source rather than retyped.  Give it the root
of a bepuphysics1 checkout:

    python oracle/extract_primes.py <path to the bepuphysics1 checkout>
"""
import re
import sys
from pathlib import Path


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/extract_primes.py <path to the bepuphysics1 checkout>")
    ref = Path(sys.argv[1])
    src = (ref / "BEPUutilities" / "PermutationMapper.cs").read_text(encoding="utf-8-sig")
    body = src[src.index("static long[] primes"):]
    body = body[body.index("{") + 1: body.index("};")]
    primes = [int(x) for x in re.findall(r"\d+", body)]
    out = Path(__file__).with_name("permutation_primes.inc")
    lines = ["// Generated by oracle/extract_primes.py from BEPUutilities/PermutationMapper.cs:49-104.",
             f"// {len(primes)} entries."]
    for i in range(0, len(primes), 8):
        lines.append("    " + ", ".join(f"{p}LL" for p in primes[i:i + 8]) + ",")
    out.write_text("\n".join(lines) + "\n")
    print(f"{len(primes)} primes -> {out}")


if __name__ == "__main__":
    main()
