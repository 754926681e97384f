"""Python binding of the C-ABI (the host-side mirror of run_SALSA).

SalsaStep(cfg) corresponds to define_salsa + salsa_initialize
(src/src_salsa/mo_salsa_init.f90:465, 792); SalsaStep.run(...) corresponds to
run_SALSA(Diag, Prog, nzp, nxp, nyp, ns, wp, pa_nactd, pa_vactd, tstep, time,
istp, level, lcharge, initialize) (src/src_salsa/mo_salsa_driver.f90:112-133)
with the Diag/Prog arrays passed as tensors (host or CUDA) in the reference
layout.  The CUDA library is required: there is no CPU path.
"""
import ctypes as C
import os

from .capi import (Config, Fields, PostFields, SedimFields, Status, make_fields, make_post_fields,
                   make_sedim_fields, ERROR_NAMES)

_lib = None


class SalsaError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what}: {ERROR_NAMES.get(code, code)} (code {code})")
        self.code = code


def library():
    """Load libsalsa_gb300.so (building it first if needed); raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    from .build import LIB, build
    if not os.path.exists(LIB):
        build()
    L = C.CDLL(LIB)
    L.salsa_gb300_default_config.argtypes = [C.POINTER(Config)]
    L.salsa_gb300_init.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.salsa_gb300_init.restype = C.c_int
    L.salsa_gb300_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                  C.c_int, C.c_int, C.c_int, C.POINTER(Fields), C.POINTER(Status)]
    L.salsa_gb300_run.restype = C.c_int
    L.salsa_gb300_run_async.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Fields), C.c_void_p, C.c_int,
                                        C.POINTER(Status)]
    L.salsa_gb300_run_async.restype = C.c_int
    L.salsa_gb300_layout.argtypes = [C.c_void_p] + [C.POINTER(C.c_int)] * 5 + [C.POINTER(C.c_double)]
    L.salsa_gb300_layout.restype = C.c_int
    L.salsa_gb300_last_launches.argtypes = [C.c_void_p]
    L.salsa_gb300_last_launches.restype = C.c_int
    L.salsa_gb300_last_kernel_ms.argtypes = [C.c_void_p]
    L.salsa_gb300_last_kernel_ms.restype = C.c_double
    L.salsa_gb300_tend_constrain.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                             C.POINTER(PostFields), C.c_void_p]
    L.salsa_gb300_tend_constrain.restype = C.c_int
    L.salsa_gb300_diagnostics.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(PostFields), C.c_void_p]
    L.salsa_gb300_diagnostics.restype = C.c_int
    L.salsa_gb300_sedimentation.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                            C.POINTER(C.c_int * 4), C.POINTER(SedimFields), C.c_void_p]
    L.salsa_gb300_sedimentation.restype = C.c_int
    L.salsa_gb300_finalize.argtypes = [C.c_void_p]
    L.salsa_gb300_version.restype = C.c_char_p
    _lib = L
    return L


EXPORTED = ["salsa_gb300_default_config", "salsa_gb300_init", "salsa_gb300_run", "salsa_gb300_run_async",
            "salsa_gb300_layout", "salsa_gb300_last_launches", "salsa_gb300_last_kernel_ms",
            "salsa_gb300_finalize", "salsa_gb300_version", "salsa_gb300_run_noalloc", "salsa_gb300_chain_state_size",
            "salsa_gb300_chain_adjoint_bytes",
            "salsa_gb300_chain_forward", "salsa_gb300_chain_tlm", "salsa_gb300_chain_adjoint",
            "salsa_gb300_tend_constrain", "salsa_gb300_diagnostics", "salsa_gb300_sedimentation"]


class SalsaStep:
    def __init__(self, cfg):
        import torch
        if not torch.cuda.is_available():
            raise SalsaError(5, "salsa_gb300_init")
        torch.cuda.init()
        self.cfg = cfg
        self.h = C.c_void_p()
        rc = library().salsa_gb300_init(C.byref(cfg), C.byref(self.h))
        if rc != 0:
            raise SalsaError(rc, "salsa_gb300_init")

    def run(self, inp, fields, outputs, time=1.0, istp=1, initialize=0, lcharge=0, stream=None, check=True):
        """One SALSA step over all interior cells of `inp` (an inputs.SalsaInputs)."""
        f = make_fields(fields, outputs)
        st = Status()
        if stream is None:
            rc = library().salsa_gb300_run(self.h, inp.nzp, inp.nxp, inp.nyp, inp.ns, inp.dt, time, istp,
                                           inp.level, lcharge, initialize, C.byref(f), C.byref(st))
        else:
            rc = library().salsa_gb300_run_async(self.h, inp.nzp, inp.nxp, inp.nyp, inp.ns, inp.dt, time, istp,
                                                 inp.level, lcharge, initialize, C.byref(f),
                                                 C.c_void_p(stream.cuda_stream), 1, C.byref(st))
        if check and rc not in (0, 4):
            raise SalsaError(rc, "salsa_gb300_run")
        return rc, st

    def layout(self):
        v = [C.c_int() for _ in range(5)]
        arr = (C.c_double * 96)()
        library().salsa_gb300_layout(self.h, *[C.byref(x) for x in v], arr)
        return [x.value for x in v], list(arr)

    def tend_constrain(self, nzp, nxp, nyp, dtlt, arrays, stream=None):
        """tend_constrain2 (src/src_LES/constrain_SALSA.f90:18-35) on CUDA tensors:
        `arrays` maps PostFields names (values and tendencies) to tensors."""
        f = make_post_fields(arrays)
        rc = library().salsa_gb300_tend_constrain(self.h, nzp, nxp, nyp, dtlt, C.byref(f),
                                                  C.c_void_p(stream.cuda_stream if stream else 0))
        if rc != 0:
            raise SalsaError(rc, "salsa_gb300_tend_constrain")

    def diagnostics(self, nzp, nxp, nyp, arrays, only_diag=0, lcharge=0, stream=None):
        """SALSA_diagnostics (src/src_LES/constrain_SALSA.f90:52-370) on CUDA tensors."""
        f = make_post_fields(arrays)
        rc = library().salsa_gb300_diagnostics(self.h, nzp, nxp, nyp, only_diag, lcharge, C.byref(f),
                                               C.c_void_p(stream.cuda_stream if stream else 0))
        if rc != 0:
            raise SalsaError(rc, "salsa_gb300_diagnostics")

    def sedimentation(self, nzp, nxp, nyp, dtlt, sed, arrays, stream=None):
        """sedim_SALSA (src/src_LES/mcrp.f90:745-905) on CUDA tensors: `arrays` maps
        SedimFields names to tensors; sed = (aero, cloud, precp, ice) switches."""
        f = make_sedim_fields(arrays)
        sw = (C.c_int * 4)(*[int(bool(x)) for x in sed])
        rc = library().salsa_gb300_sedimentation(self.h, nzp, nxp, nyp, dtlt, C.byref(sw), C.byref(f),
                                                 C.c_void_p(stream.cuda_stream if stream else 0))
        if rc != 0:
            raise SalsaError(rc, "salsa_gb300_sedimentation")

    def last_launches(self):
        return library().salsa_gb300_last_launches(self.h)

    def last_kernel_ms(self):
        return library().salsa_gb300_last_kernel_ms(self.h)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            library().salsa_gb300_finalize(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
