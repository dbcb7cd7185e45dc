"""Generate qstem_gb300/csrc/qs_rez_table.h from the reference's data header.

The electron scattering factors of Rez, Rez & Grant (Acta Cryst. A50 (1994)
481) are physical data, not code: the multislice path needs the same numbers
the reference uses (stem3/scatfactsRez.h:22-25 scatPar, :122 scatParOffs), so
this script reads them from the reference tree and re-emits them as two plain
C arrays.  Row 0 is the s-grid (1/A); row Z holds element Z.

Usage: python qstem_gb300/data/gen_rez_table.py [path/to/scatfactsRez.h]
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "..", "csrc", "qs_rez_table.h")


def parse_tables(text):
    tables = {}
    for name in ("scatPar", "scatParOffs"):
        m = re.search(r"double\s+%s\s*\[N_ELEM\]\s*\[N_SF\]\s*=\s*\{(.*?)\}\s*\}\s*;" % name, text, re.S)
        if not m:
            raise SystemExit("table %s not found" % name)
        body = m.group(1) + "}"
        rows = re.findall(r"\{([^{}]*)\}", body)
        tables[name] = [[float(v) for v in r.replace("\n", "").split(",") if v.strip()] for r in rows]
    return tables


def main():
    if len(sys.argv) > 1:
        src = sys.argv[1]
    elif os.environ.get("QS_REFERENCE_DIR"):
        src = os.path.join(os.environ["QS_REFERENCE_DIR"], "stem3", "scatfactsRez.h")
    else:
        raise SystemExit("usage: gen_rez_table.py <reference>/stem3/scatfactsRez.h "
                         "(or set QS_REFERENCE_DIR to the reference checkout)")
    with open(src) as f:
        text = f.read()
    n_elem = int(re.search(r"#define\s+N_ELEM\s+(\d+)", text).group(1))
    n_sf = int(re.search(r"#define\s+N_SF\s+(\d+)", text).group(1))
    t = parse_tables(text)
    for name, rows in t.items():
        assert len(rows) == n_elem, (name, len(rows))
        for r in rows:
            assert len(r) == n_sf, (name, len(r))
    out = []
    out.append("/* Generated by qstem_gb300/data/gen_rez_table.py -- do not edit.\n"
               " * Electron scattering factors f(s) of Rez, Rez & Grant (1994): row 0 is\n"
               " * the s-grid (1/A), row Z element Z; QS_REZ_Q holds df/dq for ions. */\n")
    out.append("#ifndef QS_REZ_TABLE_H\n#define QS_REZ_TABLE_H\n")
    out.append("#define QS_REZ_NELEM %d\n#define QS_REZ_NSF %d\n" % (n_elem, n_sf))
    for cname, key in (("QS_REZ_F", "scatPar"), ("QS_REZ_Q", "scatParOffs")):
        out.append("static const double %s[QS_REZ_NELEM][QS_REZ_NSF] = {" % cname)
        for z, r in enumerate(t[key]):
            vals = ",".join(repr(v) for v in r)
            out.append("  /* %2d */ {%s}," % (z, vals))
        out.append("};")
    out.append("#endif")
    with open(OUT, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", os.path.normpath(OUT))


if __name__ == "__main__":
    main()
