"""The ns_config drop-in (host C) against the reference parser and expected values.

Files are written by the tests (same keys and layout as the reference's
config/parameters.ini and tests/config_override.json usage in
tests/test_solvers.c:297-347).  Where the reference build (oracle/_ref) exists,
every key/value pair is compared with the reference's own parser on the same
files.
"""
import ctypes as C
import os

import pytest

import oracle as O

INI = """# solver parameters
[solver]
type = spectral

[grid]
nx = 128
ny = 128

[domain]
Lx = 2.0
Ly = 2.0

[fluid]
Re = 750.0

; time stepping
[time]
dt = 0.002
t_end = 1.5

[forcing]
type = white
energy_target = 1.25
correlation_time = 0.4

[spectral.hyperviscosity]
coefficient = 0.015
order = 8
"""

JSON = """{
  "grid": {"nx": 192, "ny": 96},
  "solver": {"type": "finite_difference"},
  "time": {"dt": 0.001},
  "extra": {"flag": true, "off": false, "none": null, "name": "a\\"b\\\\c\\/d\\n", "big": 12345678901234567890,
            "pi": 3.14159265358979323846, "neg": -1e-7}
}
"""


class Entry(C.Structure):
    _fields_ = [("key", C.c_char_p), ("value", C.c_char_p)]


class Config(C.Structure):
    _fields_ = [("entries", C.POINTER(Entry)), ("count", C.c_size_t), ("capacity", C.c_size_t)]


class SchemaEntry(C.Structure):
    _fields_ = [("key", C.c_char_p), ("type", C.c_int), ("required", C.c_int), ("min_value", C.c_double),
                ("max_value", C.c_double), ("has_min", C.c_int), ("has_max", C.c_int),
                ("allowed_values", C.POINTER(C.c_char_p)), ("allowed_count", C.c_size_t)]


def _bind(lib):
    cp = C.POINTER(Config)
    lib.ns_config_init.argtypes = [cp]
    lib.ns_config_free.argtypes = [cp]
    lib.ns_config_set.argtypes = [cp, C.c_char_p, C.c_char_p]
    lib.ns_config_get_string.restype = C.c_char_p
    lib.ns_config_get_string.argtypes = [cp, C.c_char_p, C.c_char_p]
    lib.ns_config_get_int.argtypes = [cp, C.c_char_p, C.c_int]
    lib.ns_config_get_double.restype = C.c_double
    lib.ns_config_get_double.argtypes = [cp, C.c_char_p, C.c_double]
    lib.ns_config_get_bool.argtypes = [cp, C.c_char_p, C.c_int]
    lib.ns_config_has_key.argtypes = [cp, C.c_char_p]
    lib.ns_config_load_files.argtypes = [cp, C.POINTER(C.c_char_p), C.c_size_t, C.c_char_p, C.c_size_t]
    lib.ns_config_validate.argtypes = [cp, C.POINTER(SchemaEntry), C.c_size_t, C.c_char_p, C.c_size_t]
    return lib


def _load(lib, paths):
    cfg = Config()
    lib.ns_config_init(C.byref(cfg))
    arr = (C.c_char_p * len(paths))(*[p.encode() for p in paths])
    err = C.create_string_buffer(256)
    st = lib.ns_config_load_files(C.byref(cfg), arr, len(paths), err, 256)
    return cfg, st, err.value.decode()


def _items(cfg):
    return {cfg.entries[i].key.decode(): cfg.entries[i].value.decode() for i in range(cfg.count)}


@pytest.fixture
def files(tmp_path):
    ini = tmp_path / "parameters.ini"
    js = tmp_path / "override.JSON"
    ini.write_text(INI)
    js.write_text(JSON)
    return str(ini), str(js)


@pytest.fixture(scope="module")
def product(nsgb):
    return _bind(C.CDLL(nsgb.LIB_PATH))


def test_reference_scenario(product, files):
    """tests/test_solvers.c:297-347 of the reference, restated."""
    lib = product
    cfg = Config()
    lib.ns_config_init(C.byref(cfg))
    for k, v in (("solver.type", "spectral"), ("grid.nx", "64"), ("grid.ny", "64"), ("time.dt", "0.005")):
        assert lib.ns_config_set(C.byref(cfg), k.encode(), v.encode()) == 0
    arr = (C.c_char_p * 2)(*[p.encode() for p in files])
    err = C.create_string_buffer(256)
    assert lib.ns_config_load_files(C.byref(cfg), arr, 2, err, 256) == 0, err.value
    g = lambda k, d=0: lib.ns_config_get_int(C.byref(cfg), k.encode(), d)
    gd = lambda k, d=0.0: lib.ns_config_get_double(C.byref(cfg), k.encode(), d)
    assert lib.ns_config_has_key(C.byref(cfg), b"domain.Lx")
    assert lib.ns_config_get_string(C.byref(cfg), b"solver.type", b"") == b"finite_difference"
    assert g("grid.nx") == 192 and g("grid.ny") == 96
    assert abs(gd("domain.Lx") - 2.0) < 1e-12 and abs(gd("domain.Ly") - 2.0) < 1e-12
    assert abs(gd("time.dt") - 0.001) < 1e-12
    assert abs(gd("forcing.energy_target") - 1.25) < 1e-12
    assert abs(gd("spectral.hyperviscosity.coefficient") - 0.015) < 1e-15
    solver_allowed = (C.c_char_p * 2)(b"spectral", b"finite_difference")
    forcing_allowed = (C.c_char_p * 3)(b"none", b"white", b"colored")
    S, I, D = 0, 1, 2
    rows = [
        (b"solver.type", S, 1, 0, 0, 0, 0, solver_allowed, 2), (b"grid.nx", I, 1, 2.0, 0, 1, 0, None, 0),
        (b"grid.ny", I, 1, 2.0, 0, 1, 0, None, 0), (b"domain.Lx", D, 1, 1e-6, 0, 1, 0, None, 0),
        (b"domain.Ly", D, 1, 1e-6, 0, 1, 0, None, 0), (b"fluid.Re", D, 1, 1e-6, 0, 1, 0, None, 0),
        (b"time.dt", D, 1, 1e-9, 0, 1, 0, None, 0), (b"time.t_end", D, 1, 1e-9, 0, 1, 0, None, 0),
        (b"forcing.energy_target", D, 0, 0, 0, 1, 0, None, 0), (b"forcing.type", S, 0, 0, 0, 0, 0, forcing_allowed, 3),
        (b"spectral.hyperviscosity.coefficient", D, 0, 0, 0, 1, 0, None, 0),
        (b"spectral.hyperviscosity.order", I, 0, 0, 0, 1, 0, None, 0),
    ]
    schema = (SchemaEntry * len(rows))(*[SchemaEntry(*r) for r in rows])
    assert lib.ns_config_validate(C.byref(cfg), schema, len(rows), err, 256) == 0, err.value
    # a violated bound and a forbidden string are reported
    bad = (SchemaEntry * 1)(SchemaEntry(b"grid.nx", I, 1, 500.0, 0, 1, 0, None, 0))
    assert lib.ns_config_validate(C.byref(cfg), bad, 1, err, 256) == -1
    assert b"grid.nx" in err.value
    lib.ns_config_set(C.byref(cfg), b"forcing.type", b"purple")
    assert lib.ns_config_validate(C.byref(cfg), schema, len(rows), err, 256) == -1
    lib.ns_config_free(C.byref(cfg))


def test_json_values_and_getter_fallbacks(product, files):
    lib = product
    cfg, st, err = _load(lib, [files[1]])
    assert st == 0, err
    it = _items(cfg)
    assert it["extra.flag"] == "true" and it["extra.off"] == "false" and it["extra.none"] == ""
    assert it["extra.name"] == 'a"b\\c/d\n'
    assert it["extra.big"] == "%.15g" % 12345678901234567890
    assert it["extra.pi"] == "%.15g" % 3.14159265358979323846
    assert lib.ns_config_get_bool(C.byref(cfg), b"extra.flag", 0) == 1
    assert lib.ns_config_get_bool(C.byref(cfg), b"extra.none", 7) == 7
    assert lib.ns_config_get_int(C.byref(cfg), b"time.dt", 42) == 42          # "0.001" is not an int
    assert lib.ns_config_get_double(C.byref(cfg), b"missing.key", -3.5) == -3.5
    lib.ns_config_free(C.byref(cfg))


@pytest.mark.parametrize("text,fragment", [("[grid\nnx = 1\n", "section"), ("[grid]\nnx 1\n", "key-value")])
def test_malformed_ini_reports_error(product, tmp_path, text, fragment):
    p = tmp_path / "bad.ini"
    p.write_text(text)
    cfg, st, err = _load(product, [str(p)])
    assert st == -1 and fragment in err


@pytest.mark.parametrize("text", ['{"a": 1} x', '{"a": [1, 2]}', '{"a": "unterminated}', '{"a" 1}'])
def test_malformed_json_reports_error(product, tmp_path, text):
    p = tmp_path / "bad.json"
    p.write_text(text)
    cfg, st, err = _load(product, [str(p)])
    assert st == -1 and err


def test_missing_file_reports_error(product, tmp_path):
    cfg, st, err = _load(product, [str(tmp_path / "nope.ini")])
    assert st == -1 and "Failed to open" in err


@pytest.mark.skipif(not O.have_ref(), reason="reference build not present")
def test_matches_reference_parser(product, files, tmp_path):
    O.build(ref=True)
    ref = _bind(C.CDLL(O.REF_SO))
    a, sa, _ = _load(product, list(files))
    b, sb, _ = _load(ref, list(files))
    assert sa == sb == 0
    assert _items(a) == _items(b)
    for text in ('{"a": 1} x', "[grid\n", '{"k": "v", "n": {"m": -2.5e-3}}'):
        p = tmp_path / ("c.json" if text.startswith("{") else "c.ini")
        p.write_text(text)
        x, sx, _ = _load(product, [str(p)])
        y, sy, _ = _load(ref, [str(p)])
        assert sx == sy
        if sx == 0:
            assert _items(x) == _items(y)
