"""Generate base_table.inc: constant tables compiled into the CUDA library.

  FT_BASE_COMB  32 x 8 affine entries (y+x, y-x, 2dxy) of (j+1) * 256^i * B,
                the layout of the reference's fixed-base table
                (ge25519_cmov8_base.h, used by sodium_ge.cu:480-488), recomputed
                here from the curve equation with Python integers.
  FT_L_SLIDE    signed sliding-window digits of the group order L, the
                recoding that ge25519_mul_l (sodium_ge.cu:795-847) walks.

Run:  python gen_tables.py  (rewrites base_table.inc next to this file).
"""
import os

P = 2**255 - 19
D = (-121665 * pow(121666, P - 2, P)) % P
L = 2**252 + 27742317777372353535851937790883648493
BY = 4 * pow(5, P - 2, P) % P


def xrecover(y):
    u = (y * y - 1) % P
    v = (D * y * y + 1) % P
    x2 = u * pow(v, P - 2, P) % P
    x = pow(x2, (P + 3) // 8, P)
    if (x * x - x2) % P:
        x = x * pow(2, (P - 1) // 4, P) % P
    if x & 1:
        x = P - x
    return x


BASE = (xrecover(BY), BY)


def add(a, b):
    x1, y1 = a
    x2, y2 = b
    t = D * x1 * x2 * y1 * y2 % P
    x3 = (x1 * y2 + x2 * y1) * pow(1 + t, P - 2, P) % P
    y3 = (y1 * y2 + x1 * x2) * pow(1 - t, P - 2, P) % P
    return (x3, y3)


def mul(k, pt):
    r = (0, 1)
    while k:
        if k & 1:
            r = add(r, pt)
        pt = add(pt, pt)
        k >>= 1
    return r


def words(v):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(8)]


def comb_table(q):
    rows = []
    row = q
    for i in range(32):
        acc = row
        entries = []
        for j in range(8):
            x, y = acc
            entries.append(((y + x) % P, (y - x) % P, 2 * D * x * y % P))
            acc = add(acc, row)
        rows.append(entries)
        row = mul(256, row)
    return rows


def slide(a_bytes):
    r = [1 & (a_bytes[i >> 3] >> (i & 7)) for i in range(256)]
    for i in range(256):
        if not r[i]:
            continue
        b = 1
        while b <= 6 and i + b < 256:
            if r[i + b]:
                ribs = r[i + b] << b
                if r[i] + ribs <= 15:
                    r[i] += ribs
                    r[i + b] = 0
                else:
                    if r[i] - ribs < -15:
                        break
                    r[i] -= ribs
                    for k in range(i + b, 256):
                        if not r[k]:
                            r[k] = 1
                            break
                        r[k] = 0
            b += 1
    return r


def main():
    rows = comb_table(BASE)
    out = ["// generated by gen_tables.py — do not edit",
           "// FT_BASE_COMB[i][j][c][w]: word w of coordinate c (y+x, y-x, 2dxy)",
           "// of the affine point (j+1) * 256^i * B",
           "// The includer defines FT_TABLE_QUAL (storage class and alignment).",
           "#ifdef FT_WANT_BASE_COMB",
           "FT_TABLE_QUAL uint32_t FT_BASE_COMB_INIT[32 * 8 * 3 * 8] = {"]
    for i in range(32):
        for j in range(8):
            vals = []
            for c in rows[i][j]:
                vals += ["0x%08xu" % w for w in words(c)]
            out.append("    " + ", ".join(vals) + ",")
    out.append("};")
    out.append("#endif")
    sl = slide(list(L.to_bytes(32, "little")))
    assert sum(d * 2**i for i, d in enumerate(sl)) == L
    out.append("// signed sliding-window digits of L, index 0 = least significant")
    out.append("#ifdef FT_WANT_L_SLIDE")
    out.append("FT_TABLE_QUAL signed char FT_L_SLIDE_INIT[253] = {")
    out.append("    " + ", ".join(str(d) for d in sl[:253]))
    out.append("};")
    out.append("#endif")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "base_table.inc")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path


if __name__ == "__main__":
    print(main())
