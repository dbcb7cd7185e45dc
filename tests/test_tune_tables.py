"""The autotuner's copies of the line-transform tables (qstem_gb300/tune.py)
against the sources they mirror: the factorisation lists of qs_fft.cuh and
the thread layouts qs_tuned.h sets."""
import os
import re

from qstem_gb300 import tune

CSRC = os.path.join(os.path.dirname(tune.__file__), "csrc")


def _read(name):
    with open(os.path.join(CSRC, name)) as f:
        return f.read()


def test_factorisation_lists_match_the_line_transforms():
    src = _read("qs_fft.cuh")
    for n, alts in tune.RADIX_LISTS.items():
        m = re.search(r"using Rad%d = typename pick<I,(.*?)>::type;" % n, src, re.S)
        assert m, n
        lists = [tuple(int(x) for x in g.split(",")) for g in re.findall(r"rad_t<([\d,\s]+)>", m.group(1))]
        assert lists == alts, n
        for r in lists:
            prod = 1
            for x in r:
                prod *= x
            assert prod == n


def test_thread_layouts_match_the_tuned_header():
    src = _read("qs_tuned.h")

    def define(name):
        m = re.search(r"#define %s (\w+)" % name, src)
        assert m, name
        v = m.group(1)
        return int(v) if v.isdigit() else define(v)
    for n in (384, 768):
        assert tune.ROW_T[n] == define("QS_LINE_T_%d" % n)
        assert tune.COL_T[n] == define("QS_COL_LINE_T_%d" % n)
        # the tuned factorisations fit the layouts
        assert tune.radix_ok(n, define("QS_RADIX_ROW_%d" % n))
        assert tune.radix_ok(n, define("QS_RADIX_COL_%d" % n), col=True)
    for n in (512, 1024):
        assert tune.radix_ok(n, define("QS_RADIX_ROW_%d" % n))
        assert tune.radix_ok(n, define("QS_RADIX_COL_%d" % n), col=True)
