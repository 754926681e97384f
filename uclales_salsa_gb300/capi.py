"""ctypes mirror of the C-ABI structs in include/salsa_gb300.h.

The structs restate the argument list of UCLALES-SALSA's run_SALSA
(src/src_salsa/mo_salsa_driver.f90:112-133) and the &salsa NAMELIST
(src/src_salsa/mo_salsa_init.f90:522-600); field order must match the header.
"""
import ctypes as C

MAXSPEC = 7
MAXNSP = 9
MAXBINS = 96

DIAG_NAMES = [
    "s_m_autoc", "s_m_autoc80", "s_m_autoc50", "s_m_accr", "s_m_accr80", "s_m_accr50",
    "s_m_ACcoll_dry", "s_m_APcoll_dry", "s_n_activ", "s_m_conda", "s_m_condc", "s_m_condp",
    "s_m_AIcoll_dry", "s_n_icehom", "s_n_icedep", "s_n_iceimm", "s_m_condi",
    "s_n_sipdrfr", "s_n_siprmspl", "s_n_sipiibr",
]
NDIAG = len(DIAG_NAMES)
NDIAG_LEVEL4 = 12
NDIAG_LEVEL5 = 17          # without the secondary-ice rates (lssecice off)

SALSA_OK, SALSA_E_ARG, SALSA_E_UNSUPPORTED, SALSA_E_CUDA, SALSA_E_NUMERIC, SALSA_E_NODEV = range(6)
ERROR_NAMES = {0: "ok", 1: "bad argument", 2: "unsupported configuration", 3: "CUDA error",
               4: "numerical condition (reference would STOP)", 5: "no usable GPU"}


class Switch(C.Structure):
    """ProcessSwitch (src/src_shared/classProcessSwitch.f90:5-14)."""
    _fields_ = [("sw", C.c_int), ("delay", C.c_double), ("mode", C.c_int)]


class Config(C.Structure):
    _fields_ = [
        ("level", C.c_int),
        ("lscoag", Switch), ("lscnd", Switch), ("lsauto", Switch), ("lsactiv", Switch),
        ("lsicenucl", Switch), ("lsicemelt", Switch), ("lssecice", Switch),
        ("lscgaa", C.c_int), ("lscgcc", C.c_int), ("lscgca", C.c_int), ("lscgpc", C.c_int),
        ("lscgpa", C.c_int), ("lscgpp", C.c_int), ("lscgia", C.c_int), ("lscgic", C.c_int),
        ("lscgii", C.c_int), ("lscgip", C.c_int),
        ("Eiagg_max", C.c_double), ("Eiagg_min", C.c_double),
        ("cgintvl", C.c_double),
        ("lscndgas", C.c_int), ("lscndh2oae", C.c_int), ("lscndh2ocl", C.c_int), ("lscndh2oic", C.c_int),
        ("lsicehom", C.c_int), ("lsiceimm", C.c_int), ("lsicedep", C.c_int),
        ("ice_theta_dist", C.c_int),
        ("lsFreeTheta", Switch),
        ("initMinTheta", C.c_double),
        ("mean_theta_imm", C.c_double), ("sigma_theta_imm", C.c_double),
        ("mean_theta_dep", C.c_double), ("sigma_theta_dep", C.c_double),
        ("iceShapeAlpha", C.c_double), ("iceShapeBeta", C.c_double),
        ("iceShapeGamma", C.c_double), ("iceShapeSigma", C.c_double),
        ("lsdistupdate", C.c_int),
        ("lscheckarrays", C.c_int),
        ("fixinc", C.c_double),
        ("lsfreeRH", Switch),
        ("rhlim", C.c_double),
        ("eddy_dis", C.c_double),
        ("nsnucl", C.c_int), ("nj3", C.c_int),
        ("act_coeff", C.c_double),
        ("nbin", C.c_int * 2),
        ("reglim", C.c_double * 4),
        ("prc_nbins", C.c_int), ("prc_dlo", C.c_double), ("prc_vol_ratio", C.c_double),
        ("ice_nbins", C.c_int), ("ice_dlo", C.c_double), ("ice_vol_ratio", C.c_double),
        ("nspec_dry", C.c_int),
        ("listspec", (C.c_char * 4) * MAXSPEC),
        ("chargeTMax", C.c_double), ("chargeCollEnh", C.c_double),
        ("lssiprimespln", Switch), ("lssipdropfrac", Switch), ("lssipicecollbreak", Switch),
        ("precision", C.c_int),
        ("diagnostics", C.c_int),
    ]

    def set_species(self, names):
        self.nspec_dry = len(names)
        for i in range(MAXSPEC):
            nm = names[i] if i < len(names) else ""
            self.listspec[i].value = nm.encode()

    def species(self):
        return [self.listspec[i].value.decode() for i in range(self.nspec_dry)]


_PD = C.POINTER(C.c_double)


class Fields(C.Structure):
    _fields_ = [
        ("press", _PD), ("temp", _PD), ("rsl", _PD), ("rsi", _PD), ("dn", _PD),
        ("rp", _PD), ("rpt", _PD),
        ("wp", _PD),
        ("naero", _PD), ("ncloud", _PD), ("nprecp", _PD), ("nice", _PD),
        ("naerot", _PD), ("ncloudt", _PD), ("nprecpt", _PD), ("nicet", _PD),
        ("maero", _PD), ("mcloud", _PD), ("mprecp", _PD), ("mice", _PD),
        ("maerot", _PD), ("mcloudt", _PD), ("mprecpt", _PD), ("micet", _PD),
        ("indef", _PD),
        ("chargeTime", _PD),
        ("gaero", _PD), ("gaerot", _PD),
        ("pa_nactd", _PD),
        ("pa_vactd", _PD),
        ("diag", _PD * NDIAG),
        ("kappa", _PD),
        ("sipdrfr", _PD), ("siprmspl", _PD), ("sipiibr", _PD),
    ]


SEDIM_NAMES = ("naero", "ncloud", "nprecp", "nice", "maero", "mcloud", "mprecp", "mice",
               "naerot", "ncloudt", "nprecpt", "nicet", "maerot", "mcloudt", "mprecpt", "micet",
               "tk", "th", "adn", "ustar", "dzt", "tlt", "rrate", "irate", "sfcrrate", "sfcirate", "VtPrc", "VtIce")


class PostFields(C.Structure):
    """salsa_post_fields_t: the arrays of tend_constrain2 and SALSA_diagnostics."""
    _fields_ = [(n, _PD) for n in (
        "naero", "ncloud", "nprecp", "nice", "maero", "mcloud", "mprecp", "mice", "gaero", "indef", "chargeTime",
        "naerot", "ncloudt", "nprecpt", "nicet", "maerot", "mcloudt", "mprecpt", "micet", "gaerot",
        "rh", "rhi", "temp", "rp", "rc", "srp", "snrp", "rtot", "ri", "riri")]


def make_post_fields(arrays):
    """PostFields with the data pointers of the tensors in `arrays` (name -> tensor)."""
    f = PostFields()
    names = {n for n, _ in PostFields._fields_}
    for name, t in arrays.items():
        if name not in names or t is None:
            continue
        if not t.is_contiguous() or t.dtype.itemsize != 8:
            raise ValueError(f"field {name} must be a contiguous float64 tensor")
        setattr(f, name, ptr_of(t.data_ptr()))
    return f


class SedimFields(C.Structure):
    """salsa_sedim_fields_t: the arrays of sedim_SALSA (src/src_LES/mcrp.f90:745-905)."""
    _fields_ = [(n, _PD) for n in SEDIM_NAMES]


def make_sedim_fields(arrays):
    """SedimFields with the data pointers of the tensors in `arrays` (name -> tensor)."""
    f = SedimFields()
    for name, t in arrays.items():
        if name not in SEDIM_NAMES or t is None:
            continue
        if not t.is_contiguous() or t.dtype.itemsize != 8:
            raise ValueError(f"field {name} must be a contiguous float64 tensor")
        setattr(f, name, ptr_of(t.data_ptr()))
    return f


class Status(C.Structure):
    _fields_ = [
        ("code", C.c_int),
        ("n_cells", C.c_longlong),
        ("n_equil_nonconv", C.c_longlong),
        ("n_distr_nonconv", C.c_longlong),
        ("n_distr_negfrac", C.c_longlong),
        ("n_cond_substeps", C.c_longlong),
        ("n_negative", C.c_longlong),
        ("n_nonfinite", C.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


FIELD_INPUTS = ["press", "temp", "rsl", "rsi", "dn", "rp", "wp", "naero", "ncloud", "nprecp", "nice",
                "maero", "mcloud", "mprecp", "mice", "gaero", "kappa"]
FIELD_INOUT = ["rpt", "naerot", "ncloudt", "nprecpt", "nicet", "maerot", "mcloudt", "mprecpt", "micet",
               "indef", "chargeTime", "gaerot", "pa_nactd", "pa_vactd", "sipdrfr", "siprmspl", "sipiibr"]


def ptr_of(addr):
    return C.cast(C.c_void_p(addr), _PD) if addr else _PD()


def make_fields(inputs, outputs):
    """Fill a Fields struct with the data pointers of torch tensors (host or device).

    inputs: dict name -> tensor for the read-only arrays (and indef/chargeTime,
    which are updated in place); outputs: dict of tendency/output tensors, with
    an optional "diag" tensor whose leading index is the diagnostic number."""
    f = Fields()
    for name, t in list(inputs.items()) + list(outputs.items()):
        if name == "diag":
            for i in range(min(t.shape[0], NDIAG)):
                f.diag[i] = ptr_of(t[i].data_ptr())
            continue
        if t is None:
            continue
        if not t.is_contiguous() or t.dtype.itemsize != 8:
            raise ValueError(f"field {name} must be a contiguous float64 tensor")
        setattr(f, name, ptr_of(t.data_ptr()))
    return f
