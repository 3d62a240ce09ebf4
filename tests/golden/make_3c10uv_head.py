"""Generate tests/golden/3c10uv_head.fts: the first NGROUPS groups of the reference's
reqdata/3C10UV.FTS (VLA random-groups data, 32-bit integers with PSCALn/BSCALE) with its
GCOUNT card rewritten to NGROUPS and the data padded to a whole 2880-byte block.  The
header is otherwise byte for byte the reference's, so the GPU loader can be checked on the
reference's own file format where the reference tree is absent; the expected values are the
first NGROUPS entries of tests/golden/3c10.npz (made by make_3c10.py from the whole file).

Usage: python tests/golden/make_3c10uv_head.py [path/to/reqdata]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NGROUPS = 300



def reference_root():
    """The reference tree: $SDE_REFERENCE, else /root/reference (None if that is not an
    existing directory)."""
    root = os.environ.get("SDE_REFERENCE") or "/root/reference"
    return root if os.path.isdir(root) else None

def main(reqdata):
    raw = open(os.path.join(reqdata, "3C10UV.FTS"), "rb").read()
    cards, i = [], 0
    while True:
        card = raw[i:i + 80]
        i += 80
        if card[:8] == b"GCOUNT  ":
            card = b"GCOUNT  = %20d /" % NGROUPS
            card = card + b" " * (80 - len(card))
        cards.append(card)
        if card[:3] == b"END":
            break
    off = (i + 2879) // 2880 * 2880
    head = b"".join(cards)
    head += b" " * (off - len(head))
    npar = 6
    lgrp = npar + 3 * 4
    data = raw[off:off + NGROUPS * lgrp * 4]
    assert len(data) == NGROUPS * lgrp * 4
    data += b"\0" * ((-len(data)) % 2880)
    out = os.path.join(HERE, "3c10uv_head.fts")
    open(out, "wb").write(head + data)
    print("wrote", out, len(head) + len(data), "bytes")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        root = reference_root()
        if root is None:
            sys.exit("no reference tree: pass path/to/reqdata or set SDE_REFERENCE")
        main(os.path.join(root, "reqdata"))
