"""CPU tests of the C-ABI library: it loads, exports what the header declares, and its
structs have the layout the ctypes mirror assumes.  No compute calls (no GPU here)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from uclales_salsa_gb300 import api, capi
from uclales_salsa_gb300.chain import ChainDesc
from uclales_salsa_gb300.config import reference_defaults, workload_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "salsa_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(salsa_gb300_\w+)\s*\(", txt)))


def test_library_exports_every_declared_entry_point():
    lib = api.library()
    names = declared_functions()
    assert set(names) == set(api.EXPORTED)
    for n in names:
        assert hasattr(lib, n), n
    assert lib.salsa_gb300_version().startswith(b"salsa_gb300")


def _offsets_from_c(struct, fields):
    src = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', 'int main(void){']
    src.append(f'printf("%zu\\n", sizeof({struct}));')
    for f in fields:
        src.append(f'printf("%zu\\n", offsetof({struct}, {f}));')
    src.append('return 0;}')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(x) for x in out]


@pytest.mark.parametrize("struct,cls", [("salsa_config_t", capi.Config), ("salsa_fields_t", capi.Fields),
                                        ("salsa_status_t", capi.Status), ("salsa_chain_t", ChainDesc)])
def test_struct_layout_matches_ctypes(struct, cls):
    fields = [n for n, _ in cls._fields_]
    got = _offsets_from_c(struct, fields)
    assert got[0] == C.sizeof(cls)
    for n, off in zip(fields, got[1:]):
        assert getattr(cls, n).offset == off, n


def test_default_config_matches_reference_defaults():
    c = capi.Config()
    api.library().salsa_gb300_default_config(C.byref(c))
    r = reference_defaults(5)
    for name, _ in capi.Config._fields_:
        a, b = getattr(c, name), getattr(r, name)
        if isinstance(a, capi.Switch):
            assert (a.sw, a.delay, a.mode) == (b.sw, b.delay, b.mode), name
        elif name == "listspec":
            assert c.species() == r.species()
        elif hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name


def test_null_arguments_are_rejected():
    lib = api.library()
    h = C.c_void_p()
    assert lib.salsa_gb300_init(None, C.byref(h)) == capi.SALSA_E_ARG
    st = capi.Status()
    assert lib.salsa_gb300_run(None, 42, 20, 20, 6, 1.0, 1.0, 1, 4, 0, 0, None, C.byref(st)) == capi.SALSA_E_ARG


def test_secondary_ice_modes_outside_the_reference_are_refused_before_any_device_call():
    """salsa_gb300_init answers SALSA_E_UNSUPPORTED, before it touches a device, for the
    secondary-ice modes the reference does not define (rime splintering outside 1-2, drop
    fracturing outside 1-4, ice-ice breakup outside 1-3); every mode it defines gets past
    that check."""
    lib = api.library()
    h = C.c_void_p()
    for scheme, modes in (("lssiprimespln", (0, 3)), ("lssipdropfrac", (0, 5)), ("lssipicecollbreak", (0, 4))):
        for mode in modes:
            cfg = reference_defaults(level=5)
            cfg.lssecice.sw = 1
            sw = getattr(cfg, scheme)
            sw.sw, sw.mode = 1, mode
            assert lib.salsa_gb300_init(C.byref(cfg), C.byref(h)) == capi.SALSA_E_UNSUPPORTED, (scheme, mode)
    for scheme, modes in (("lssiprimespln", (1, 2)), ("lssipdropfrac", (1, 2, 3, 4)), ("lssipicecollbreak", (1, 2, 3))):
        for mode in modes:
            # the 7-bin precipitation and ice layout of the workloads: on a GPU, init goes on
            # to size the shared memory, which the secondary-ice form with the 20-bin
            # default layout exceeds (also SALSA_E_UNSUPPORTED)
            cfg = workload_config(5)
            cfg.lssecice.sw = 1
            sw = getattr(cfg, scheme)
            sw.sw, sw.mode = 1, mode
            rc = lib.salsa_gb300_init(C.byref(cfg), C.byref(h))
            assert rc != capi.SALSA_E_UNSUPPORTED, (scheme, mode)
            if rc == capi.SALSA_OK:
                lib.salsa_gb300_finalize(h)
    cfg = reference_defaults(level=5)
    rc = lib.salsa_gb300_init(C.byref(cfg), C.byref(h))
    assert rc != capi.SALSA_E_UNSUPPORTED
    if rc == capi.SALSA_OK:
        lib.salsa_gb300_finalize(h)
    cfg = reference_defaults(level=5)
    rc = lib.salsa_gb300_init(C.byref(cfg), C.byref(h))
    assert rc != capi.SALSA_E_UNSUPPORTED
    if rc == capi.SALSA_OK:
        lib.salsa_gb300_finalize(h)
