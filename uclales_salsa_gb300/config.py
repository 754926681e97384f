"""Configuration builders for the SALSA step (the &salsa NAMELIST as a C struct).

reference_defaults() restates the module defaults of the reference
(src/src_shared/mo_submctl.f90:19-160, mo_ice_shape.f90:25-30,
classProcessSwitch.f90:5-14, mo_salsa_init.f90:687-695 setDefaultBinLayouts).

workload_config(level) is the switch set of the measured workloads: the
runles-style &salsa block (bin/runles_dcc:244-379) with every coagulation
sub-process on, coagulation-based precipitation formation (lsauto mode 1),
interstitial activation (lsactiv mode 1), immersion freezing with the
contact-angle distribution, 17 aerosol bins (3 in 1a, 7 in 2a, 7 in 2b) between
3 nm and 10 um, 7 precipitation bins spanning 20 um - 2 mm, 7 ice bins from 2 um
with volume ratio 3, and species SO4 OC BC DU SS.
"""
from .capi import Config, Switch


def _sw(c, on, delay=0.0, mode=1):
    c.sw, c.delay, c.mode = int(on), float(delay), int(mode)


def reference_defaults(level=5):
    c = Config()
    c.level = level
    for name in ("lscoag", "lscnd", "lsauto", "lsactiv", "lsicenucl", "lsicemelt", "lssecice",
                 "lsFreeTheta", "lsfreeRH", "lssiprimespln", "lssipdropfrac", "lssipicecollbreak"):
        _sw(getattr(c, name), False)
    for name in ("lscgaa", "lscgcc", "lscgca", "lscgpc", "lscgpa", "lscgpp", "lscgia", "lscgic",
                 "lscgii", "lscgip"):
        setattr(c, name, 1)
    c.Eiagg_max, c.Eiagg_min = 0.3, 0.05
    c.cgintvl = 10.0
    c.lscndgas, c.lscndh2oae, c.lscndh2ocl, c.lscndh2oic = 0, 1, 1, 1
    c.lsicehom = c.lsiceimm = c.lsicedep = 0
    c.ice_theta_dist = 1
    c.initMinTheta = 0.0
    c.mean_theta_imm, c.sigma_theta_imm = 132.0, 20.0
    c.mean_theta_dep, c.sigma_theta_dep = 15.5, 1.4
    c.iceShapeAlpha, c.iceShapeBeta, c.iceShapeGamma, c.iceShapeSigma = 15.56999e-3, 2.02, 0.55, 1.97
    c.lsdistupdate = 1
    c.lscheckarrays = 0
    c.fixinc = -1.0
    c.rhlim = 1.20
    c.eddy_dis = 0.001
    c.nsnucl, c.nj3 = 0, 1
    c.act_coeff = 1.e-7
    c.nbin[0], c.nbin[1] = 3, 8
    for i, v in enumerate((3.e-9, 4.e-8, 7.e-7, 1.5e-5)):
        c.reglim[i] = v
    c.prc_nbins, c.prc_dlo, c.prc_vol_ratio = 20, 20.e-6, 2.0
    c.ice_nbins, c.ice_dlo, c.ice_vol_ratio = 20, 20.e-6, 2.0
    c.set_species(["SO4"])
    c.chargeTMax, c.chargeCollEnh = 1000.0, 0.0
    c.precision = 0
    c.diagnostics = 1
    return c


def workload_config(level=5, precision=0, diagnostics=1):
    c = reference_defaults(level)
    for name in ("lscoag", "lscnd", "lsauto", "lsactiv"):
        _sw(getattr(c, name), True)
    _sw(c.lsicenucl, level == 5)
    _sw(c.lsicemelt, level == 5)
    _sw(c.lssecice, False)
    _sw(c.lsFreeTheta, True, 0.0)
    _sw(c.lsfreeRH, True, 0.0)
    c.lsiceimm = 1 if level == 5 else 0
    c.nbin[0], c.nbin[1] = 3, 7
    for i, v in enumerate((3.e-9, 4.e-8, 7.e-7, 1.e-5)):
        c.reglim[i] = v
    c.prc_nbins, c.prc_dlo, c.prc_vol_ratio = 7, 20.e-6, 100.0 ** (3.0 / 7.0)
    c.ice_nbins, c.ice_dlo, c.ice_vol_ratio = 7, 2.e-6, 3.0
    c.set_species(["SO4", "OC", "BC", "DU", "SS"])
    c.precision = precision
    c.diagnostics = diagnostics
    return c


def config_dict(c):
    out = {}
    for name, _ in Config._fields_:
        v = getattr(c, name)
        if isinstance(v, Switch):
            v = {"switch": v.sw, "delay": v.delay, "mode": v.mode}
        elif name == "listspec":
            v = c.species()
        elif hasattr(v, "__len__"):
            v = list(v)
        out[name] = v
    return out
