"""Benchmark of the GB300 SALSA step (one JSON line on rank 0).

A step is one SALSA call over every interior cell of the workload
(run_SALSA, src/src_salsa/mo_salsa_driver.f90:112-435).  Default workload: the
384x384x160 grid (23,592,960 cells), level 5, dt = 1 s, 10 % cloudy cells in
convective columns with ice, the other 90 % clear at RH 40-85 %.  Its fields (about
158 GB) stay resident on the device; the steps read them in place (the IN deficit,
the only input a step rewrites, is put back before the error and end-to-end legs).

  value  -- FP64 (parity) form, cell-steps/s, inputs resident in HBM, CUDA events on
            the launch stream around exactly K steps (after W warm-up steps).
  mixed  -- the FP32-mixed form on the same inputs, and its per-field error against
            the FP64 form over every interior cell (one step of each from one state).
  e2e    -- FP64 form through the C-ABI with page-locked HOST buffers: the host->device
            copy of every array and the device->host copy of the results are inside
            the timed region (the C-ABI moves them in y-slabs that overlap the
            computation).  The buffers are one exactly sized allocation registered with
            the driver; the leg is skipped, with a note, when the host lacks the memory.
  roofline -- algorithmic bytes per cell-step (8 * (3S + T + G + I + A + D)) over the
            measured HBM copy bandwidth; the step is FP64-pipe bound, so the fraction is
            small and the ncu FP64 pipe figures are in profiles/.
  cpu_baseline -- the FP64 CPU oracle (a C restatement of the reference path; the
            Fortran cannot be built here) on a bounded sample, all host threads, and on
            a smaller sample with one thread; the CPU model from lscpu.
  post_step -- tend_constrain2, SALSA_diagnostics and sedim_SALSA over the grid.
  adjoint -- forward and adjoint time of the gradient harness (65,536 warm cells, 60
            coagulation + condensation steps of 0.5 s, checkpoints every step).

--impl reference times that CPU implementation alone on bounded samples of the same
workload.  With torchrun, every rank runs the workload on its own GPU (independent
cells, no collective on the data path); value is the sum over ranks of the cells
over the slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

# algorithmic doubles per cell-step: prog read + tendency RMW (3S), thermo + rv RMW (T),
# gases (G), IN deficit R+W (I), activation outputs (A), diagnostics (D)
ALG_DOUBLES = {4: 3 * 266 + 8 + 5 + 0 + 98 + 12, 5: 3 * 322 + 9 + 5 + 76 + 98 + 17}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def field_bytes(d):
    return sum(v.numel() * v.element_size() for v in d.values())


def host_buffers(sources):
    """Host copies of `sources` (name -> tensor to copy, or torch.Size of a zeroed array) in
    one exactly sized host allocation registered with the CUDA driver (page-locked).
    torch's pinned allocator rounds every block up to a power of two, which would take up
    to twice the host memory for the largest workload."""
    import torch
    shape = {k: (v.shape if isinstance(v, torch.Tensor) else torch.Size(v)) for k, v in sources.items()}
    total = sum(math.prod(x) for x in shape.values())
    buf = torch.zeros(total, dtype=torch.float64)
    rc = torch._C._cudart.cudaHostRegister(buf.data_ptr(), total * 8, 0)
    if int(rc) != 0:
        raise RuntimeError(f"cudaHostRegister failed ({rc})")
    out, off = {}, 0
    for k, v in sources.items():
        n = math.prod(shape[k])
        view = buf[off:off + n].view(shape[k])
        if isinstance(v, torch.Tensor):
            view.copy_(v)
        out[k] = view
        off += n
    return buf, out


def mem_available_bytes():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def form_errors(inp, fields, out_a, out_b, tol=1e-6):
    """Per-field relative error of the new state x = old + tendency * dt of form b against
    form a, over every interior cell, on the device: max, RMS and the fraction within tol.
    The scale of a bin value is max(|x_a|, |old|, floor) with the parity tests' floors."""
    import torch
    from parity import STATE_OF, floor_of, interior
    res = {}
    for name, st in STATE_OF.items():
        if name not in out_a or name not in out_b:
            continue
        n, s2, mx, over = 0, 0.0, 0.0, 0
        for b in range(out_a[name].shape[0] if out_a[name].dim() == 4 else 1):
            pick = (lambda t: t[b]) if out_a[name].dim() == 4 else (lambda t: t)
            I = lambda t: interior(pick(t), inp.nzp, inp.nxp, inp.nyp)
            old = I(fields[st])
            xa, xb = old + I(out_a[name]) * inp.dt, old + I(out_b[name]) * inp.dt
            scale = torch.maximum(xa.abs(), old.abs()).clamp(min=floor_of(name))
            rel = (xb - xa).abs() / scale
            n += rel.numel()
            s2 += float((rel * rel).sum())
            mx = max(mx, float(rel.max()))
            over += int((rel > tol).sum())
        res[name] = {"max": mx, "rms": (s2 / n) ** 0.5, "frac_within_1e-6": 1.0 - over / n}
    return res


def run_gb300(args):
    import torch
    import torch.distributed as tdist
    from uclales_salsa_gb300.inputs import make_inputs, make_outputs
    from uclales_salsa_gb300.api import SalsaStep
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        tdist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            tdist.barrier()
        torch.cuda.synchronize()

    def tmax(x):
        t = torch.tensor([x], device=dev)
        if world > 1:
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        return float(t.item())

    inp = make_inputs(args.workload, dev, precision=0, diagnostics=1)
    ncell = inp.ncells
    level = inp.level
    fields = inp.fields           # the steps read the workload's fields; only the IN deficit changes
    indef0 = fields["indef"].clone() if "indef" in fields else None

    def restore():
        if indef0 is not None:
            fields["indef"].copy_(indef0)

    results = {}
    stream = torch.cuda.Stream(device=dev)
    outs = make_outputs(inp)
    for form in (0, 1):
        inp.cfg.precision = form
        step = SalsaStep(inp.cfg)
        warm = args.warmup if form == 0 else min(args.warmup, 3)
        for _ in range(warm):
            step.run(inp, fields, outs, time=1.0, stream=stream)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kms = []
        nlaunch = 0
        sampler = ClockSampler(local) if form == 0 else None
        if sampler:
            sampler.__enter__()
        barrier()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.steps):
                step.run(inp, fields, outs, time=1.0, stream=stream)
                kms.append(step.last_kernel_ms())
                nlaunch += step.last_launches()
            e1.record(stream)
        barrier()
        if sampler:
            sampler.__exit__()
            results["clocks"] = sampler.summary()
        results[form] = dict(ms_total=tmax(e0.elapsed_time(e1)), kernel_ms=sum(kms) / len(kms), launches=nlaunch,
                             warmup=warm)
        step.close()
    del outs
    torch.cuda.empty_cache()

    # mixed form against the FP64 form: one step of each from the same state
    errors = None
    if not args.no_errors:
        res = {}
        for form in (0, 1):
            inp.cfg.precision = form
            restore()
            o = make_outputs(inp, with_diag=False)
            step = SalsaStep(inp.cfg)
            step.run(inp, fields, o, time=1.0, stream=stream)
            torch.cuda.synchronize()
            step.close()
            res[form] = o
        restore()
        errors = form_errors(inp, fields, res[0], res[1])
        del res
        torch.cuda.empty_cache()
    inp.cfg.precision = 0

    # bytes a step moves across the boundary: the C-ABI copies the interior y rows
    # (nyp - 4 of nyp) of every array it uses in, outputs included (so that their
    # values outside the interior cells come back unchanged), and of the tendencies,
    # outputs and IN deficit back out
    outs_meta = make_outputs(inp, device="meta")
    rows = (inp.nyp - 4) / inp.nyp
    inputs_b = sum(v.numel() * 8 for k, v in fields.items() if k in (
        "press", "temp", "rsl", "rsi", "rp", "dn", "wp", "naero", "ncloud", "nprecp", "nice", "maero", "mcloud",
        "mprecp", "mice", "indef"))
    indef_b = fields["indef"].numel() * 8 if "indef" in fields else 0
    h2d = int(round((inputs_b + field_bytes(outs_meta)) * rows))
    d2h = int(round((field_bytes(outs_meta) + indef_b) * rows))
    e2e_s, e2e_note, e2e_warm = None, None, min(args.warmup, 3)
    if not args.no_e2e:
        # end to end through the C-ABI with page-locked host buffers (FP64 form)
        need = field_bytes(fields) + field_bytes(outs_meta)
        avail = mem_available_bytes()
        if avail < need + 24 * 2 ** 30:
            e2e_note = f"skipped: {need / 1e9:.0f} GB of host buffers, {avail / 1e9:.0f} GB available"
        else:
            restore()
            src = dict(fields)
            src.update({"out_" + k: v.shape for k, v in outs_meta.items()})
            buf, host = host_buffers(src)
            host_in = {k: v for k, v in host.items() if not k.startswith("out_")}
            host_out = {k[4:]: v for k, v in host.items() if k.startswith("out_")}
            del src
            step = SalsaStep(inp.cfg)
            for _ in range(e2e_warm):
                step.run(inp, host_in, host_out, time=1.0)   # the first call allocates the staging slots
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                step.run(inp, host_in, host_out, time=1.0)
            barrier()
            e2e_s = tmax(time.perf_counter() - t0)
            step.close()
            torch._C._cudart.cudaHostUnregister(buf.data_ptr())
            del host_in, host_out, host, buf
    else:
        e2e_note = "not measured (--no-e2e)"

    post = None
    if not args.no_post:
        step = SalsaStep(inp.cfg)
        outs = make_outputs(inp)
        step.run(inp, fields, outs, time=1.0, stream=stream)
        post = post_bench(step, inp, fields, outs, stream, peak_gbs())   # changes the fields (last use)
        step.close()
        del outs
        torch.cuda.empty_cache()

    r0 = results[0]
    value = world * ncell * args.steps / (r0["ms_total"] / 1e3)
    mixed = world * ncell * args.steps / (results[1]["ms_total"] / 1e3)
    e2e = world * ncell * args.steps / e2e_s if e2e_s else None
    bytes_cell = 8 * ALG_DOUBLES[level]
    peak, peak_src = peak_gbs()
    achieved = bytes_cell * ncell / (r0["kernel_ms"] / 1e3) / 1e9
    # DRAM bytes per cell and FP64-pipe activity from the committed ncu capture of the step
    # kernel on a block of this workload, scaled to the cells of one launch (ncu cannot run
    # inside the timed region)
    traffic, fp64_pipe, tsrc = None, None, None
    tp = os.path.join(ROOT, "profiles", "salsa_step_kernel.json")
    if os.path.exists(tp):
        try:
            prof = json.load(open(tp))[args.workload]
            traffic = prof["dram_bytes_per_cell"]["fp64"] * ncell
            fp64_pipe = prof["fp64_pipe_active_pct"]
            tsrc = prof["source"]
        except Exception:
            traffic = None
    line = {
        "metric": "cell-steps/s (FP64 SALSA step; FP32-mixed form in 'mixed')",
        "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r0["ms_total"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, run_SALSA layout)",
        "config": {"workload": args.workload, "cells": ncell, "level": level, "dt_s": inp.dt,
                   "l2": "inputs larger than L2 (%.1f GB per step)" % ((h2d + d2h) / 1e9)},
        "mixed": {"value": mixed, "unit": "cell-steps/s", "ms_per_step": results[1]["ms_total"] / args.steps,
                  "warmup": results[1]["warmup"], "speedup_vs_fp64": mixed / value,
                  "dtype": "f32 collision kernels, mass-transfer coefficients and pair sums + f64 state",
                  "errors_vs_fp64": errors,
                  "errors_note": "one step of each form from the same state, every interior cell; relative to "
                                 "max(|x_fp64|, |x_old|, floor) of the new state x = old + tendency * dt"},
        "e2e": ({"value": e2e, "unit": "cell-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                 "warmup": e2e_warm, "host_buffers": "page-locked (cudaHostRegister), one allocation"}
                if e2e is not None else {"value": None, "note": e2e_note}),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": tsrc, "peak_source": peak_src,
                     "algorithmic_bytes_per_cell": bytes_cell,
                     "note": "the step is bound by the FP64 pipe, not HBM",
                     "fp64_pipe_active_pct_ncu": fp64_pipe},
        "gpu_launches": r0["launches"],
        "clocks": results.get("clocks"),
    }
    if post:
        line["post_step"] = post
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = chain_bench(dev)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_sample_cells)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()


def peak_gbs():
    """HBM copy bandwidth: the measured peak, else the fallback figure."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def post_bench(step, inp, fields, outs, stream, peak, reps=3):
    """tend_constrain2, SALSA_diagnostics and sedim_SALSA over the whole grid after the
    timed steps (fields and tendencies resident): device time per call and HBM roofline
    fraction of the bytes each call must read or write.  The sedimentation is bound by
    the FP64 pipe (fall speeds), not by HBM."""
    from uclales_salsa_gb300.post_case import (post_arrays, post_bytes, time_post, sedim_arrays, sedim_bytes,
                                               time_sedim)
    a = post_arrays(inp, fields, outs)
    tc_ms, dg_ms = time_post(step, inp, a, stream, reps)
    tcb, dgb = post_bytes(a, inp.level)
    del a
    sa = sedim_arrays(inp, fields, outs)
    sd_ms = time_sedim(step, inp, sa, stream, reps)
    sdb = sedim_bytes(sa)
    del sa
    return {"what": "tend_constrain2 + SALSA_diagnostics (constrain_SALSA.f90) and sedim_SALSA (mcrp.f90) over "
                    "the grid, fields in HBM",
            "tend_constrain_ms": tc_ms, "diagnostics_ms": dg_ms, "sedimentation_ms": sd_ms,
            "tend_constrain": {"bytes": tcb, "achieved_gbs": tcb / tc_ms / 1e6,
                               "frac": tcb / tc_ms / 1e6 / peak[0]},
            "diagnostics": {"bytes": dgb, "achieved_gbs": dgb / dg_ms / 1e6, "frac": dgb / dg_ms / 1e6 / peak[0]},
            "sedimentation": {"bytes": sdb, "achieved_gbs": sdb / sd_ms / 1e6, "frac": sdb / sd_ms / 1e6 / peak[0],
                              "bound": "fp64",
                              "setup": "all four parts, 20 m levels, ustar 0.3 m/s, dtlt = step"},
            "peak_gbs": peak[0], "peak_source": peak[1]}


def chain_bench(dev, nsub=60):
    """Forward and adjoint time of the gradient harness on its workload: 65,536 warm
    cells, nsub coagulation + condensation steps of 0.5 s, checkpoints every step."""
    import torch
    from uclales_salsa_gb300.inputs import make_inputs
    from uclales_salsa_gb300.chain import SalsaChain, chain_config, pack_state
    inp = make_inputs("chain65536", dev)
    inp.cfg = chain_config()
    x, th, k, s = pack_state(inp)
    ch = SalsaChain(inp.cfg)
    yb = torch.zeros_like(x)
    lay = inp.layout
    nl = lay.nbins + lay.ncld + lay.nprc
    for b in range(lay.nbins, lay.nbins + lay.ncld):   # loss: final cloud numbers and masses
        yb[:, b] = 1.0
        for sp in range(lay.nwet):
            yb[:, nl + sp * nl + b] = 1.0
    xw, ckw = ch.forward(x, th, k, s, 2, inp.dt)          # warm-up (module load, allocation)
    ch.adjoint(ckw, 1, th, k, s, 2, inp.dt, yb)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    ev[0].record()
    xN, ck = ch.forward(x, th, k, s, nsub, inp.dt, ckpt_every=1)
    ev[1].record()
    xb, kb, sb = ch.adjoint(ck, 1, th, k, s, nsub, inp.dt, yb / xN.abs().clamp(min=1e-30))
    ev[2].record()
    torch.cuda.synchronize()
    f_ms, a_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    ch.close()
    return {"workload": f"chain65536 ({x.shape[0]} cells, {nsub} steps of {inp.dt} s, coagulation + condensation)",
            "forward_ms": f_ms, "adjoint_ms": a_ms, "adjoint_over_forward": a_ms / f_ms, "checkpoint_every": 1,
            "gradients_finite": bool(torch.isfinite(xb).all() and torch.isfinite(kb).all() and torch.isfinite(sb).all())}


def oracle_sample(workload, cells):
    """A cubic-ish sub-block of the workload with the same distributions."""
    from uclales_salsa_gb300.inputs import WORKLOADS, make_inputs
    spec = WORKLOADS[workload]
    Z = min(spec["Z"], 32)
    side = max(1, int(round((cells / Z) ** 0.5)))
    return make_inputs(workload, "cpu", X=side, Y=side, Z=Z)


def cpu_model():
    """The host CPU's model name (lscpu), e.g. Neoverse-V2 on the GB300 hosts."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


def cpu_baseline(workload, cells, single_core_cells=32768):
    """The FP64 oracle on a sample of the workload with every host thread, and on a
    smaller sample with one thread."""
    from uclales_salsa_gb300.inputs import make_outputs
    from oracle_ref import Oracle
    res = {}
    for n, threads in ((cells, 0), (single_core_cells, 1)):
        inp = oracle_sample(workload, n)
        o = Oracle(inp.cfg)
        f = {k: v.clone() for k, v in inp.fields.items()}
        out = make_outputs(inp)
        t0 = time.perf_counter()
        o.run(inp, f, out, time=1.0, nthreads=threads)
        res[threads] = (inp, time.perf_counter() - t0)
        del f, out
    inp, dt = res[0]
    inp1, dt1 = res[1]
    return {"value": inp.ncells / dt, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{inp.ncells} cells ({inp.nxp - 4}x{inp.nyp - 4}x{inp.nzp - 2}) of {workload}, FP64 oracle, "
                      f"{dt:.1f} s",
            "single_core": {"value": inp1.ncells / dt1, "unit": "cell-steps/s",
                            "sample": f"{inp1.ncells} cells ({inp1.nxp - 4}x{inp1.nyp - 4}x{inp1.nzp - 2}), "
                                      f"{dt1:.1f} s"}}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from uclales_salsa_gb300.inputs import make_outputs
    from oracle_ref import Oracle
    inp = oracle_sample(args.workload, args.cpu_sample_cells)
    o = Oracle(inp.cfg)
    times = []
    for i in range(args.warmup + args.steps):
        f = {k: v.clone() for k, v in inp.fields.items()}
        out = make_outputs(inp)
        t0 = time.perf_counter()
        o.run(inp, f, out, time=1.0)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    value = inp.ncells * len(times) / sum(times)
    sample = (f"{inp.ncells} cells ({inp.nxp - 4}x{inp.nyp - 4}x{inp.nzp - 2}) of {args.workload} per step; "
              "FP64 C restatement of the reference path (the Fortran reference cannot be built: no Fortran compiler)")
    line = {"impl": "reference", "metric": "cell-steps/s (FP64 SALSA step; FP32-mixed form in 'mixed')",
            "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * inp.ncells / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, run_SALSA layout)",
            "config": {"workload": args.workload, "cells_per_step": inp.ncells},
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": os.cpu_count(), "kind": "port",
                             "cpu_model": cpu_model(), "sample": sample},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="grid384x384x160")
    ap.add_argument("--cpu-sample-cells", type=int, default=3145728)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-post", action="store_true", help="skip the tend_constrain2 / SALSA_diagnostics timing")
    ap.add_argument("--no-errors", action="store_true", help="skip the mixed-vs-FP64 error block")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg through host buffers")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
