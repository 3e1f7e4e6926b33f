"""Regenerate ``mc_tables.inc`` from the reference's marching-cubes tables.

The triangle table has to be the same table, entry for entry, as the one the
reference uses (``modules/include/cuda/marching_cubes_tables.cuh:93``): the
order of the triangles of a cube and of the edges of a triangle fixes the
order of the emitted vertices, which the compatibility mode reproduces bit for
bit.  The table itself is the classic Lorensen–Cline case table in the layout
published by Cory Bloyd (public domain); the reference ships it under MIT.

This script stores it in a different, denser form:

* ``GBT_MC_TRI_PACKED[256]`` — one 64-bit word per cube case; edge ``k`` of
  the case's triangle list sits in bits ``[4k, 4k+4)``.
* ``GBT_MC_TRI_COUNT[256]`` — triangles per case (0..5).
* ``GBT_MC_EDGE_ENDS[12]`` — start corner in the low nibble, end corner in the
  high nibble (the start/end order matters for the interpolation rule).
* ``GBT_MC_EDGE_MASK[256]`` — the 12-bit set of intersected edges, derived
  from the triangle list and checked here against the reference's own edge
  table (``marching_cubes_tables.cuh:18``).

Run it from the repository root, naming the reference checkout (argument or
``REFERENCE_ROOT``):
``python cu-reconstruction_gb300/csrc/gen_mc_tables.py <reference checkout>``.
"""
import os
import re
import sys


def _array_body(text, name):
    m = re.search(name + r"\s*(\[[^\]]*\])+\s*=\s*\{", text)
    if not m:
        raise SystemExit("table %s not found" % name)
    i = m.end()
    depth = 1
    j = i
    while depth:
        c = text[j]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        j += 1
    return text[i:j - 1]


def _ints(body):
    return [int(tok, 0) for tok in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]


def load_reference_tables(ref_root):
    path = os.path.join(ref_root, "modules/include/cuda/marching_cubes_tables.cuh")
    with open(path) as f:
        text = f.read()
    text = re.sub(r"//[^\n]*", "", text)
    edge_vertices = _ints(_array_body(text, "MC_EDGE_VERTICES"))
    edge_table = _ints(_array_body(text, "MC_EDGE_TABLE"))
    tri_flat = _ints(_array_body(text, "MC_TRI_TABLE"))
    assert len(edge_vertices) == 24 and len(edge_table) == 256 and len(tri_flat) == 256 * 16
    ends = [(edge_vertices[2 * e], edge_vertices[2 * e + 1]) for e in range(12)]
    tri = [tri_flat[16 * c:16 * c + 16] for c in range(256)]
    return ends, edge_table, tri


def pack(ends, edge_table, tri):
    packed, counts, masks = [], [], []
    for c in range(256):
        row = tri[c]
        n = 0
        while n < 15 and row[n] != -1:
            n += 1
        assert n % 3 == 0 and all(v == -1 for v in row[n:]), c
        word = 0
        mask = 0
        for k in range(n):
            word |= (row[k] & 0xF) << (4 * k)
            mask |= 1 << row[k]
        packed.append(word)
        counts.append(n // 3)
        masks.append(mask)
        # the intersected-edge set derived from the triangles must equal the
        # reference's edge table and the set of sign-changing edges
        assert mask == edge_table[c], (c, hex(mask), hex(edge_table[c]))
        sign = [(c >> v) & 1 for v in range(8)]
        geo = sum(1 << e for e in range(12) if sign[ends[e][0]] != sign[ends[e][1]])
        assert geo == mask, c
    return packed, counts, masks


def emit(packed, counts, masks, ends):
    out = []
    out.append("// Generated by gen_mc_tables.py -- do not edit.")
    out.append("// Marching-cubes case tables (Lorensen-Cline cases, triangle order of the")
    out.append("// public-domain table by Cory Bloyd as used by cu-Reconstruction, MIT).")
    out.append("// Packed: edge k of a case's triangle list in bits [4k,4k+4) of a u64.")
    out.append("#define GBT_MC_TABLE_DATA \\")
    out.append("GBT_MC_CONST unsigned char GBT_MC_EDGE_ENDS[12] = {%s}; \\" %
               ", ".join("0x%02x" % (s | (e << 4)) for s, e in ends))
    for name, vals, fmt, per in (
            ("unsigned char GBT_MC_TRI_COUNT[256]", counts, "%d", 32),
            ("unsigned short GBT_MC_EDGE_MASK[256]", masks, "0x%03x", 16),
            ("unsigned long long GBT_MC_TRI_PACKED[256]", packed, "0x%015xull", 4)):
        out.append("GBT_MC_CONST %s = { \\" % name)
        for i in range(0, 256, per):
            out.append("  " + ", ".join(fmt % v for v in vals[i:i + per]) + ", \\")
        out.append("}; \\")
    out.append("")
    return "\n".join(out) + "\n"


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT")
    if not ref_root:
        sys.exit("usage: gen_mc_tables.py <reference checkout>  (or set REFERENCE_ROOT)")
    ends, edge_table, tri = load_reference_tables(ref_root)
    packed, counts, masks = pack(ends, edge_table, tri)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mc_tables.inc")
    with open(dst, "w") as f:
        f.write(emit(packed, counts, masks, ends))
    print("wrote", dst)


if __name__ == "__main__":
    main()
