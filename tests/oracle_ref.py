"""ctypes access to the CPU oracle (oracle/salsa_ref.c) for the tests.

The oracle is test infrastructure: it is loaded only by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg.
"""
import ctypes as C
import os
import subprocess

from uclales_salsa_gb300.capi import (Config, Fields, PostFields, SedimFields, Status, make_fields,
                                     make_post_fields, make_sedim_fields)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "libsalsa_ref.so")
# the same restatement built with multiply-add contraction (see oracle/Makefile)
LIB_CONTRACT = os.path.join(ROOT, "oracle", "_build", "libsalsa_ref_contract.so")
_libs = {}


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


def lib(variant="plain"):
    if variant not in _libs:
        path = LIB if variant == "plain" else LIB_CONTRACT
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        L.salsa_ref_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
        L.salsa_ref_create.restype = C.c_int
        L.salsa_ref_destroy.argtypes = [C.c_void_p]
        L.salsa_ref_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Fields), C.POINTER(Status),
                                    C.c_int, C.c_int]
        L.salsa_ref_run.restype = C.c_int
        L.salsa_ref_layout.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 5 + [C.POINTER(C.c_double)]
        L.salsa_ref_counters.argtypes = [C.c_void_p, C.POINTER(C.c_longlong * 5)]
        L.salsa_ref_states.argtypes = [C.c_void_p, C.POINTER(C.c_int * 12)]
        L.salsa_ref_terminal_vel.argtypes = [C.c_double] * 5 + [C.c_int]
        L.salsa_ref_terminal_vel.restype = C.c_double
        L.salsa_ref_nucleation_rate.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
        L.salsa_ref_nucleation_rate.restype = C.c_double
        L.salsa_ref_freezing_fraction.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 7
        L.salsa_ref_freezing_fraction.restype = C.c_double
        L.salsa_ref_sweq.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double), C.c_double]
        L.salsa_ref_sweq.restype = C.c_double
        L.salsa_ref_coagc_pair.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_double] * 6
        L.salsa_ref_coagc_pair.restype = C.c_double
        L.salsa_ref_coagc_sections.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double), C.c_int,
                                               C.c_double, C.POINTER(C.c_double), C.c_double, C.c_double]
        L.salsa_ref_coagc_sections.restype = C.c_double
        L.salsa_ref_ice_shape.argtypes = [C.c_void_p] + [C.c_double] * 3 + [C.POINTER(C.c_double * 5)]
        L.salsa_ref_tend_constrain.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                               C.POINTER(PostFields)]
        L.salsa_ref_tend_constrain.restype = C.c_int
        L.salsa_ref_diagnostics.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(PostFields)]
        L.salsa_ref_diagnostics.restype = C.c_int
        L.salsa_ref_sedimentation.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                              C.POINTER(C.c_int * 4), C.POINTER(SedimFields)]
        L.salsa_ref_sedimentation.restype = C.c_int
        L.salsa_ref_set_libm_perturbation.argtypes = [C.c_int]
        _libs[variant] = L
    return _libs[variant]


class Oracle:
    """variant "plain" is the parity oracle (no multiply-add contraction); "contract" is
    the same source built with contraction, used only for the parity envelope."""

    def __init__(self, cfg, variant="plain"):
        self.cfg = cfg
        self.variant = variant
        self.L = lib(variant)
        self.h = C.c_void_p()
        rc = self.L.salsa_ref_create(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"salsa_ref_create failed: {rc}")

    def run(self, inp, fields, outputs, time=1.0, istp=1, initialize=0, lcharge=0, nthreads=0, carry_over=0,
            libm=0):
        """libm != 0 moves every library-function result by one ulp for this run
        (salsa_ref_set_libm_perturbation)."""
        f = make_fields(fields, outputs)
        st = Status()
        self.L.salsa_ref_set_libm_perturbation(libm)
        try:
            rc = self.L.salsa_ref_run(self.h, inp.nzp, inp.nxp, inp.nyp, inp.ns, inp.dt, time, istp, inp.level,
                                      lcharge, initialize, C.byref(f), C.byref(st), nthreads, carry_over)
        finally:
            self.L.salsa_ref_set_libm_perturbation(0)
        return rc, st

    def tend_constrain(self, nzp, nxp, nyp, dtlt, arrays):
        f = make_post_fields(arrays)
        return self.L.salsa_ref_tend_constrain(self.h, nzp, nxp, nyp, dtlt, C.byref(f))

    def diagnostics(self, nzp, nxp, nyp, arrays, only_diag=0, lcharge=0):
        f = make_post_fields(arrays)
        return self.L.salsa_ref_diagnostics(self.h, nzp, nxp, nyp, only_diag, lcharge, C.byref(f))

    def sedimentation(self, nzp, nxp, nyp, dtlt, sed, arrays):
        f = make_sedim_fields(arrays)
        sw = (C.c_int * 4)(*[int(bool(x)) for x in sed])
        return self.L.salsa_ref_sedimentation(self.h, nzp, nxp, nyp, dtlt, C.byref(sw), C.byref(f))

    def layout(self):
        v = [C.c_int() for _ in range(5)]
        arr = (C.c_double * 96)()
        self.L.salsa_ref_layout(self.h, *[C.byref(x) for x in v], arr)
        return [x.value for x in v], list(arr)

    def counters(self):
        a = (C.c_longlong * 5)()
        self.L.salsa_ref_counters(self.h, C.byref(a))
        return list(a)

    def states(self):
        """Process states of set_SALSA_runtime, in the order of salsa_ref_states."""
        a = (C.c_int * 12)()
        self.L.salsa_ref_states(self.h, C.byref(a))
        names = ("lscoag", "lscnd", "lsauto", "lsactiv", "lsicenucl", "lsicemelt", "lssecice", "lssiprimespln",
                 "lssipdropfrac", "lssipicecollbreak", "lsfreeRH", "lsFreeTheta")
        return dict(zip(names, list(a)))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.salsa_ref_destroy(self.h)
            self.h = None
