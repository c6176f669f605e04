"""Generate base_table.inc: constant tables compiled into the CUDA library.

  FT_L_SLIDE    signed sliding-window digits of the group order L, the
                recoding that ge25519_mul_l (sodium_ge.cu:795-847) walks.

(The fixed-base comb tables are built on the device from B and the public
key, k_encrypt.cu.)

Run:  python gen_tables.py  (rewrites base_table.inc next to this file).
"""
import os

L = 2**252 + 27742317777372353535851937790883648493


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
    out = ["// generated by gen_tables.py — do not edit",
           "// The includer defines FT_TABLE_QUAL (storage class and alignment)."]
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
