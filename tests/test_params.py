"""The .par reader of the library against the reference's parsing rules
(src/parameter.c:13-98): same values on the reference's fixtures and on edge
cases (tabs, missing comments, prefix matches, repeated keys), and the
extension keys. Host logic only: no GPU needed."""
from __future__ import annotations

import ctypes as C

import pytest

FIELDS = ["imax", "jmax", "kmax", "xlength", "ylength", "zlength", "itermax", "eps", "omg",
          "re", "tau", "gamma", "te", "dt", "gx", "gy", "gz", "name", "bcLeft", "bcRight",
          "bcBottom", "bcTop", "bcFront", "bcBack", "u_init", "v_init", "w_init", "p_init",
          "levels", "presmooth", "postsmooth"]

DCAVITY_TEXT = """\
# driven cavity
name dcavity        # name of flow setup
bcLeft    1\t\t\t#  flags
bcRight   1\t\t\t#
bcBottom  1\t\t\t#
bcTop     1\t\t\t#
bcFront   1\t\t\t#
bcBack    1\t\t\t#
gx    0.0\t\t\t#
gy    0.0\t\t\t#
gz    0.0\t\t\t#
re    1000.0\t\t# Reynolds number
u_init    0.0\t\t#
v_init    0.0\t\t#
w_init    0.0\t\t#
p_init    0.0\t\t#
xlength    1.0\t\t#
ylength    1.0\t\t#
zlength    1.0\t\t#
imax       128\t\t#
jmax       128\t\t#
kmax       128\t\t#
te       10.0\t\t#
dt       0.02\t    #
tau      0.5\t\t#
levels        2         #
presmooth     50        #
postsmooth    5         #
itermax  1000\t\t#
eps      0.001\t\t#
omg      1.8\t\t#
gamma    0.9\t\t#
"""

EDGE_TEXT = """\
name canal
imax\t77
jmax 33 44
kmax  12
retry 5.5
re 250
tau 0.25
tau 0.75
eps 1e-7 # tolerance
omg
gammaX 0.5
bcTopX 3
u_init -1.5e-2 #
"""


def _parse(lib, path):
    from nusif import abi
    p = abi.Parameter()
    lib.initParameter(C.byref(p))
    lib.readParameter(C.byref(p), str(path).encode())
    return {f: getattr(p, f) for f in FIELDS}


def _ref_parse(path):
    import oracle
    from nusif import abi
    lib = C.CDLL(str(oracle._ref_path("rb", False)))
    p = abi.Parameter()
    lib.refdrv_read_parameter.argtypes = [C.c_char_p, C.c_void_p]
    assert lib.refdrv_sizeof_parameter() == C.sizeof(abi.Parameter)
    lib.refdrv_read_parameter(str(path).encode(), C.byref(p))
    return {f: getattr(p, f) for f in FIELDS}


@pytest.mark.parametrize("text", [DCAVITY_TEXT, EDGE_TEXT], ids=["dcavity", "edge"])
def test_parser_matches_reference(nusif_lib, tmp_path, text):
    import oracle
    if not oracle.ref_available("rb"):
        pytest.skip("reference not compiled here")
    path = tmp_path / "case.par"
    path.write_text(text)
    mine = _parse(nusif_lib, path)
    ref = _ref_parse(path)
    # fields the file leaves unset are uninitialised in both: compare the set ones
    for k in FIELDS:
        if k in text or k in ("xlength", "ylength", "zlength", "imax", "jmax", "kmax",
                              "itermax", "eps", "omg", "re", "gamma", "tau", "levels",
                              "presmooth", "postsmooth"):
            assert mine[k] == ref[k], k


def test_parser_rules_without_reference(nusif_lib, tmp_path):
    path = tmp_path / "edge.par"
    path.write_text(EDGE_TEXT)
    v = _parse(nusif_lib, path)
    assert v["name"] == b"canal\n"      # no comment after the value: newline kept
    assert v["imax"] == 100              # "imax\t77" is one token: default stays
    assert v["jmax"] == 33               # only the first value counts
    assert v["kmax"] == 12
    assert v["re"] == 250.0              # "retry 5.5" set re first, "re 250" later
    assert v["tau"] == 0.75              # later lines win
    assert v["eps"] == 1e-7
    assert v["omg"] == 1.7               # no value: default stays
    assert v["gamma"] == 0.5             # prefix match: "gammaX" sets gamma
    assert v["bcTop"] == 3
    assert v["u_init"] == -1.5e-2


def test_dcavity_fixture_values(nusif_lib, tmp_path):
    path = tmp_path / "dcavity.par"
    path.write_text(DCAVITY_TEXT)
    v = _parse(nusif_lib, path)
    assert v["name"] == b"dcavity"
    assert (v["imax"], v["jmax"], v["kmax"]) == (128, 128, 128)
    assert (v["te"], v["dt"], v["tau"], v["omg"], v["eps"]) == (10.0, 0.02, 0.5, 1.8, 0.001)
    assert (v["levels"], v["presmooth"], v["postsmooth"], v["itermax"]) == (2, 50, 5, 1000)


def test_write_par_round_trip(nusif_lib, tmp_path):
    from nusif.params import channel, write_par
    vals = channel(imax=40, jmax=10, kmax=10)
    path = write_par(tmp_path / "ch.par", vals)
    v = _parse(nusif_lib, path)
    for k in FIELDS:
        if k in vals:
            want = vals[k].encode() if isinstance(vals[k], str) else vals[k]
            assert v[k] == want, k


def test_extension_keys(nusif_lib, tmp_path):
    from nusif import abi
    p = abi.Parameter()
    nusif_lib.initParameter(C.byref(p))
    for k, val in [("solver", "mg-mixed"), ("lid", "1.5"), ("inflow", "1.0"), ("rtol", "1e-8"),
                   ("mg_levels", "5"), ("mg_pre", "3"), ("mg_post", "1"), ("mg_inner", "3"),
                   ("mg_theta", "0.9"), ("mg_omega", "1.2"), ("mg_chunk", "8"),
                   ("mg_guess", "quadratic"), ("mg_guess", "cubic"), ("mg_tail", "0"),
                   ("host_fields", "1"),
                   ("mg_probe", "8"), ("fg_arith", "fp64"), ("fg_arith", "df32"),
                   ("arith", "fp64"), ("arith", "df32"), ("fuse_dt", "1")]:
        assert nusif_lib.nusifParameterSet(C.byref(p), k.encode(), val.encode()) == 0
    # extension keys do not disturb the reference members
    assert p.levels == 5 and p.presmooth == 5 and p.re == 100.0
