"""H·psi benchmark: determinant updates per second of one restricted
two-body apply on the norb=14, (7 alpha, 7 beta) sector (3432 x 3432 =
11,778,624 determinants, complex128), seeded synthetic integrals with 28
Cholesky vectors.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                  [--precision auto|fp64|ozaki]

One step = one apply sigma = H psi over the whole sector.  `value` is timed
with the inputs resident in HBM (psi is 188 MB and the dvec blocks tens of GB,
both larger than the 129 MB L2); `e2e` times the same apply through the C ABI
entry fqegpu_apply_host with pinned host buffers (host->device copy of psi and
device->host copy of sigma inside the timed region).  Under torchrun every
rank runs an independent replica (the path does not shard); rank 0 prints.

The second half of the metric, Davidson time to a 1e-6 residual with the
learned vs the plain diagonal preconditioner, is the "davidson" object of the
same line (default sector norb=12 (6a,6b); --davidson-norb, --no-davidson).

  python bench.py --configs      the other single-GPU configurations (norb 8
                                 apply and Taylor step; norb 14 FP64 vs
                                 tensor-core error, Taylor, diagonal-Coulomb
                                 evolve), one JSON object
  python bench.py --norb 16 --precision ozaki --no-davidson
                                 the 165.6 M-determinant sector
  python bench.py --batch        256 uneven sectors (norb 8-12): apply and Taylor
                                 graphs, default vs autotuned launch shape
  python bench.py --taylor16     20 Taylor steps dt=0.05 at norb 16 (8a,8b) on
                                 the tensor cores, first step against FP64
  python bench.py --no-cpu-baseline --davidson-norb 16 --davidson-scratch-gb 20
                                 Davidson to 1e-6 at norb 16, learned vs plain
  python bench.py --diag         the norb-14 diagonal-Coulomb evolve, 20 calls
  python bench.py --rdm          the norb-14 one- and two-particle RDMs
  python bench.py --rows         spin-orbital apply (norb 12), orbital rotation
                                 and save/read (norb 14)
"""

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "openfermion-fqe_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

NORB, NALPHA, NBETA, NCHOL, SEED = 14, 7, 7, 28, 0
METRIC = ("H*psi det-updates/s at norb=14; Davidson time-to-1e-6 resid, "
          "learned vs plain")


def set_workload(norb, nalpha, nbeta, nchol):
    """Other sector sizes, for profiling captures on a smaller case."""
    global NORB, NALPHA, NBETA, NCHOL, METRIC
    NORB, NALPHA, NBETA, NCHOL = norb, nalpha, nbeta, nchol
    METRIC = f"H*psi det-updates/s at norb={norb}"
UNIT = "det/s"
# the tensor-core contraction: BF16 slices of D (psi's digits) and products
OZ_DSLICES, OZ_PRODUCTS = 6, 20
# DRAM bytes of one k_oz_fused launch over its algorithmic bytes, from a full
# ncu capture of the norb-12 bench command (psi's digit planes fit in L2
# there), used for sizes without a capture of their own
FUSED_TRAFFIC_RATIO = 1.03
# measured DRAM bytes (read, write) of one k_oz_fused launch by norb for the
# half-filled sector: one-pass ncu counters (dram__bytes_read.sum,
# dram__bytes_write.sum) on the bench command itself
FUSED_TRAFFIC_MEASURED = {14: (13.69e9, 19.74e9)}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed
    region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        top = max(sm) if sm else 0.0
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """Largest per-rank timing over the job (the job is as slow as its slowest
    replica); the identity for one rank."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(n_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job determinant updates per second: every replica applies its own
    full sector (weak scaling)."""
    return world * n_per_rank / seconds


def make_inputs():
    from fqe_gb300 import synthetic
    return synthetic.sector(NORB, NALPHA, NBETA, NCHOL, SEED)


def cpu_apply_time(h1, h2, psi, threads):
    """One apply of the oracle port (the reference algorithm restated in C,
    OpenMP over `threads` host threads)."""
    import oracle
    oracle.build()
    oracle.set_threads(threads)
    g = oracle.graph(NORB, NALPHA, NBETA)
    t0 = time.perf_counter()
    oracle.apply_spatial12(psi, h1, h2, g)
    return time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    h1, h2, psi = make_inputs()
    n = psi.size
    for _ in range(args.warmup):
        cpu_apply_time(h1, h2, psi, cores)
    times = [cpu_apply_time(h1, h2, psi, cores) for _ in range(args.steps)]
    t = sum(times) / len(times)
    value = n / t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"restricted H*psi, norb={NORB} ({NALPHA}a,{NBETA}b), "
                               f"{NCHOL} Cholesky vectors, seed {SEED}", "norb": NORB,
                   "nalpha": NALPHA, "nbeta": NBETA, "determinants": n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores,
                         "kind": "port",
                         "sample": f"full norb={NORB} apply per step (the reference "
                                   "C algorithm restated in oracle/fqe_oracle.c,"
                                   " OpenMP)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import numpy
    import torch
    import torch.distributed as dist
    import fqe_gb300
    from fqe_gb300 import _lib, settings
    from fqe_gb300.fqe_data import ham_for, _ptr

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    settings._device_index = local
    if world > 1:
        dist.init_process_group("nccl")
    fqe_gb300.build()

    h1, h2, psi_h = make_inputs()
    n = psi_h.size
    prec = args.precision
    if prec == "auto":
        prec = "fp64"
        try:
            settings.precision = "ozaki"
            d0 = fqe_gb300.FqeData(2, 2, 4)
            d0.set_wfn(strategy="ones")
            d0.apply((numpy.eye(4), numpy.zeros((4,) * 4)))
            prec = "ozaki"
        except NotImplementedError:
            pass
        finally:
            settings.precision = "fp64"
    settings.precision = prec
    pcode = settings.precision_code()

    d = fqe_gb300.FqeData(NALPHA, NBETA, NORB)
    d.set_wfn(strategy="from_data", raw_data=psi_h)
    ham = ham_for(d._core, h1, h2)
    sigma = torch.empty_like(d.coeff)
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.call("fqegpu_apply", ham.handle, _ptr(d.coeff), _ptr(sigma),
                  1.0, 0.0, 0.0, 0.0, pcode, sptr)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 0)):
        step()
    barrier()
    _lib.call("fqegpu_ham_set_timing", ham.handle, 1)
    stage = numpy.zeros(3)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    # per-stage times: one more timed pass per step would perturb the timed
    # region, so the stage split is read from the last timed apply
    s3 = numpy.zeros(3)
    _lib.call("fqegpu_ham_stage_ms", ham.handle,
              s3.ctypes.data_as(ctypes.c_void_p))
    stage[:] = s3
    _lib.call("fqegpu_ham_set_timing", ham.handle, 0)
    # the applies are asynchronous: a tensor-core timeout would be reported here
    _lib.call("fqegpu_ham_check", ham.handle, sptr)
    clocks = clk.summary()
    # error of the timed result against the FP64 GPU apply (validated against
    # the oracle by the tests), computed once outside the timed region
    rel_err = None
    if prec != "fp64":
        sigma64 = torch.empty_like(sigma)
        _lib.call("fqegpu_apply", ham.handle, _ptr(d.coeff), _ptr(sigma64),
                  1.0, 0.0, 0.0, 0.0, _lib.PREC_FP64, sptr)
        torch.cuda.synchronize()
        rel_err = float(torch.linalg.norm(sigma - sigma64) / torch.linalg.norm(sigma64))
        del sigma64

    t_max = max_over_ranks(ms, world)
    value = job_value(n, world, t_max / 1e3)

    # e2e: host buffers through the C ABI (pinned)
    psi_pin = torch.from_numpy(psi_h).pin_memory()
    out_pin = torch.empty_like(psi_pin).pin_memory()

    def step_e2e():
        _lib.call("fqegpu_apply_host", ham.handle,
                  ctypes.c_void_p(psi_pin.data_ptr()),
                  ctypes.c_void_p(out_pin.data_ptr()), 1.0, 0.0, 0.0, 0.0, pcode)

    step_e2e()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    # correctness guard on the e2e output (cheap: norm of sigma vs device run)
    e2e_ok = bool(numpy.isfinite(out_pin.numpy()).all())

    P = ham.npairs
    lena = d.lena()
    hbm_peak, bf16_peak, peak_src = peaks()
    flops_fp64_peak = 1.10  # TFLOP/s, GB300 DGEMM measured with torch (float64 matmul)
    # algorithmic work per apply (contraction: 2 real GEMMs of
    # P x P x N; gather writes and scatter reads D/G at 16 B per element)
    KP = (P + 15) // 16 * 16
    if prec == "ozaki":
        # stage "gather": the digit pre-pass (k_oz_rowexp reads psi, k_oz_digits
        # reads psi and writes the 24-byte digit words); stage "contraction":
        # k_oz_fused (gathers the digits from L2, forms D in shared memory,
        # 20 useful BF16 products of P x P x (2 real columns), writes G)
        contract_flops = OZ_PRODUCTS * 2.0 * P * P * 2.0 * n
        gather_bytes = 16.0 * n + 16.0 * n + 24.0 * n
    else:
        contract_flops = 2.0 * 2.0 * P * P * n
        gather_bytes = 16.0 * n + 16.0 * P * n
    scatter_bytes = 16.0 * P * n + 16.0 * n
    names = ["gather", "contraction", "scatter"]
    dom = int(numpy.argmax(stage))
    if prec == "ozaki":
        roof_c = {"bound": "tensor", "peak": bf16_peak, "unit": "TFLOP/s"}
    else:
        roof_c = {"bound": "fp64", "peak": flops_fp64_peak, "unit": "TFLOP/s"}
    stages = {
        "gather": {"ms": stage[0], "bound": "hbm", "unit": "GB/s",
                   "achieved": gather_bytes / (stage[0] / 1e3) / 1e9 if stage[0] else None,
                   "peak": hbm_peak},
        "contraction": dict(roof_c, ms=stage[1],
                            achieved=contract_flops / (stage[1] / 1e3) / 1e12 if stage[1] else None),
        "scatter": {"ms": stage[2], "bound": "hbm", "unit": "GB/s",
                    "achieved": scatter_bytes / (stage[2] / 1e3) / 1e9 if stage[2] else None,
                    "peak": hbm_peak},
    }
    dk = stages[names[dom]]
    traffic = None
    traffic_src = None
    if prec == "ozaki" and names[dom] == "contraction":
        # k_oz_fused DRAM bytes per launch: measured at this size where a
        # one-pass capture exists, else the norb-12 full capture's ratio to
        # the algorithmic bytes (psi's digit words read once, G written
        # once) scaled to this workload
        meas = FUSED_TRAFFIC_MEASURED.get(NORB) if NALPHA == NBETA == NORB // 2 else None
        if meas:
            traffic = meas[0] + meas[1]
            traffic_src = (f"ncu one-pass capture at norb {NORB}: dram read {meas[0] / 1e9:.2f} GB"
                           f" + write {meas[1] / 1e9:.2f} GB")
        else:
            traffic = FUSED_TRAFFIC_RATIO * (24.0 * n + 16.0 * P * n)
            traffic_src = "ncu capture at norb 12 scaled by algorithmic bytes"
    roofline = {"kernel": names[dom], "bound": dk["bound"],
                "achieved": dk["achieved"], "peak": dk["peak"],
                "unit": dk["unit"],
                "frac": (dk["achieved"] / dk["peak"]) if dk["achieved"] else None,
                "traffic": traffic,
                "traffic_source": traffic_src,
                "peak_source": peak_src if dk["bound"] != "fp64"
                else "torch float64 matmul 4096^3 on a GB300"}
    # whole-apply HBM view with the uncompressed dvec byte model 16 norb^2 + 32
    alg_bytes = (16.0 * NORB * NORB + 32.0) * n
    apply_hbm = {"bytes_per_det": 16 * NORB * NORB + 32,
                 "achieved_gbs": alg_bytes / (ms / 1e3) / 1e9,
                 "peak_gbs": hbm_peak,
                 "frac": alg_bytes / (ms / 1e3) / 1e9 / hbm_peak}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        t_cpu = cpu_apply_time(h1, h2, psi_h, cores)
        cpu = {"value": n / t_cpu, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"one full norb={NORB} apply of the oracle port "
                         f"(reference C algorithm restated, OpenMP) took {t_cpu:.2f} s"}

    if prec == "ozaki":
        launches_per_apply = 5  # rowexp, globalexp, digits, fused, scatter
    else:
        launches_per_apply = 3 * math.ceil(d.lenb() / max(1, _block_w(ham)))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else "bf16-slices/f32-acc/f64",
        "data": "synthetic",
        "config": {"workload": f"restricted H*psi, norb={NORB} ({NALPHA}a,{NBETA}b), "
                               f"{NCHOL} Cholesky vectors, seed {SEED}", "norb": NORB,
                   "nalpha": NALPHA,
                   "nbeta": NBETA, "determinants": n, "precision": prec,
                   "pairs": P, "compressed_pairs": bool(ham.compressed),
                   "l2": "inputs larger than L2 (psi 188 MB; D and G blocks "
                         f"{2 * 16 * P * n / 1e9:.1f} GB)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": job_value(n, world, e2e_s), "unit": UNIT,
                "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n,
                "finite": e2e_ok},
        "gpu_launches": launches_per_apply * args.steps,
        "roofline": roofline,
        "stages": stages,
        "apply_hbm_view": apply_hbm,
        "rel_err_vs_fp64": rel_err,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0 and world == 1 and not args.no_davidson:
        # the headline sector's handles and buffers are released first: the
        # Davidson subspace of a large sector needs the device memory
        from fqe_gb300.fqe_data import clear_ham_cache
        del ham, d, sigma, psi_pin, out_pin
        clear_ham_cache()
        import gc
        gc.collect()
        torch.cuda.empty_cache()
        line["davidson"] = davidson_leg(args.davidson_norb, args.davidson_subspace,
                                        args.davidson_scratch_gb,
                                        args.davidson_max_iter, prec)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def davidson_leg(norb, subspace=32, scratch_gb=None, max_iter=400,
                 precision="ozaki", verbose=False):
    """Davidson to a 1e-6 residual on one sector, plain diagonal vs learned
    preconditioner, same GPU, same seeded synthetic integrals, applies in
    `precision` ("ozaki": tensor cores, "fp64")."""
    import torch
    import fqe_gb300
    from fqe_gb300 import davidson as dav, precond, synthetic
    na, nb = norb // 2, norb - norb // 2
    nchol = synthetic.default_nchol(norb)
    h1, h2, _ = synthetic.integrals(norb, nchol, SEED)
    ham = fqe_gb300.RestrictedHamiltonian((h1, h2))
    kw = dict(block=4, tol=1e-6, max_subspace=subspace, max_iter=max_iter,
              precision=precision, verbose=verbose,
              scratch_limit=None if scratch_gb is None else int(scratch_gb * 2**30))
    # warm-up of both arms: plans, tables, caches, the inference kernel
    dav.davidson(ham, na, nb, **dict(kw, max_iter=2))
    pre = None
    if os.path.exists(precond.DEFAULT_WEIGHTS):
        pre = precond.LearnedPreconditioner.load()
        dav.davidson(ham, na, nb, preconditioner=pre, **dict(kw, max_iter=2))
    torch.cuda.synchronize()

    def row(r, extra=None):
        d = {"seconds": r.seconds, "iterations": r.iterations,
             "applies": r.applies, "energy": float(r.eigenvalues[0]),
             "converged": bool(r.converged),
             "final_residual": float(r.residual_history[-1][0])}
        d.update(extra or {})
        return d

    plain = dav.davidson(ham, na, nb, **kw)
    out = {"workload": f"lowest root, norb={norb} ({na}a,{nb}b), {nchol} "
                       f"Cholesky vectors, seed {SEED}; block 4, subspace <= {subspace},"
                       f" residual 1e-6, {precision} applies",
           "plain": row(plain), "learned": None}
    if pre is not None:
        learned = dav.davidson(ham, na, nb, preconditioner=pre, **kw)
        out["learned"] = row(learned, {
            "rejected_learned_vectors": learned.learned_rejected,
            "switched_to_plain_at_iteration": learned.fallback_iteration})
        out["energy_difference"] = float(learned.eigenvalues[0]
                                         - plain.eigenvalues[0])
        out["time_ratio_learned_over_plain"] = learned.seconds / plain.seconds
    else:
        out["note"] = "no trained preconditioner weights in the package"
    return out


def configs_leg():
    """The benchmark's other single-GPU configurations, measured once each on
    their seeded synthetic inputs (CUDA events on the current stream):
    norb 8 (4a,4b) one apply and a Taylor step t = 0.05 to 1e-12; norb 14
    (7a,7b) FP64 vs tensor-core apply (relative error), a diagonal-Coulomb
    evolve t = 0.1 (V ~ N(0, 0.5) symmetric) and a Taylor step t = 0.05 to
    1e-12 on both paths (relative error, norm)."""
    import numpy
    import torch
    import fqe_gb300
    from fqe_gb300 import settings, synthetic

    def timed(fn, reps=1):
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            r = fn()
        e.record()
        torch.cuda.synchronize()
        return r, s.elapsed_time(e) / reps

    def wfn(norb, na, nb, psi):
        w = fqe_gb300.Wavefunction([[na + nb, na - nb, norb]])
        w.set_wfn(strategy="from_data", raw_data={(na + nb, na - nb): psi})
        return w

    def rel(a, b):
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))

    old = settings.precision
    out = {}
    try:
        settings.precision = "fp64"
        h1, h2, psi = synthetic.sector(8, 4, 4, synthetic.default_nchol(8), SEED)
        ham = fqe_gb300.RestrictedHamiltonian((h1, h2))
        w = wfn(8, 4, 4, psi)
        w.apply(ham)
        _, t_ap = timed(lambda: w.apply(ham), 20)
        w.apply_generated_unitary(0.05, "taylor", ham, accuracy=1e-12, expansion=80)
        ev, t_ev = timed(lambda: w.apply_generated_unitary(
            0.05, "taylor", ham, accuracy=1e-12, expansion=80))
        out["norb8_fp64"] = {"apply_ms": t_ap, "taylor_ms": t_ev,
                             "taylor_terms": ev._taylor_terms,
                             "taylor_norm": float(torch.linalg.norm(ev.get_coeff((8, 0))))}

        norb, na, nb = 14, 7, 7
        key = (na + nb, na - nb)
        h1, h2, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), SEED)
        ham = fqe_gb300.RestrictedHamiltonian((h1, h2))
        w = wfn(norb, na, nb, psi)
        row = {}
        res = {}
        for prec in ("fp64", "ozaki"):
            settings.precision = prec
            w.apply(ham)
            s, t_ap = timed(lambda: w.apply(ham), 3)
            ev, t_ev = timed(lambda: w.apply_generated_unitary(
                0.05, "taylor", ham, accuracy=1e-12, expansion=80))
            res[prec] = (s.get_coeff(key), ev.get_coeff(key))
            row[prec] = {"apply_ms": t_ap, "taylor_ms": t_ev,
                         "taylor_terms": ev._taylor_terms,
                         "taylor_norm": float(torch.linalg.norm(ev.get_coeff(key)))}
        row["apply_rel_err_ozaki_vs_fp64"] = rel(res["ozaki"][0], res["fp64"][0])
        row["taylor_rel_err_ozaki_vs_fp64"] = rel(res["ozaki"][1], res["fp64"][1])
        settings.precision = "fp64"
        dc = fqe_gb300.get_diagonalcoulomb_hamiltonian(synthetic.diagonal_coulomb(norb, SEED))
        w.time_evolve(0.1, dc, inplace=True)
        _, t_dc = timed(lambda: w.time_evolve(0.1, dc, inplace=True), 10)
        n = psi.size
        row["diag_coulomb_evolve"] = {
            "ms": t_dc, "gbs": 32.0 * n / (t_dc / 1e3) / 1e9,
            "norm_after_11_steps": float(torch.linalg.norm(w.get_coeff(key)))}
        # one- and two-particle RDMs of the sector (FqeData.rdm12): the
        # dvecs' Gram matrix streamed by k_rdm2_gram, norb^4 N complex MACs
        # in FP64 over the Hermitian half
        d = w._civec[key]
        d.rdm12()
        _, t_r12 = timed(lambda: d.rdm12())
        _, t_r1 = timed(lambda: d.rdm1(), 3)
        p = norb * norb
        row["rdm"] = {"rdm1_ms": t_r1, "rdm12_ms": t_r12,
                      "rdm12_fp64_tflops": 8.0 * p * (p + 1) / 2 * n / (t_r12 / 1e3) / 1e12}
        out["norb14"] = row
    finally:
        settings.precision = old
    return out


def diag_leg(norb=14, calls=20):
    """The diagonal-Coulomb evolve t = 0.1 of the norb (norb/2, norb/2)
    sector (V ~ N(0, 0.5) symmetric, seeded), in place, `calls` times (CUDA
    events on the current stream): time per call, its 32 B/det against the
    measured copy rate, and the norm afterwards."""
    import torch
    import fqe_gb300
    from fqe_gb300 import settings, synthetic
    na = nb = norb // 2
    key = (na + nb, 0)
    _, _, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), SEED)
    w = fqe_gb300.Wavefunction([[na + nb, 0, norb]])
    w.set_wfn(strategy="from_data", raw_data={key: psi})
    dc = fqe_gb300.get_diagonalcoulomb_hamiltonian(synthetic.diagonal_coulomb(norb, SEED))
    old = settings.precision
    try:
        settings.precision = "fp64"
        for _ in range(3):
            w.time_evolve(0.1, dc, inplace=True)
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(calls):
            w.time_evolve(0.1, dc, inplace=True)
        e.record()
        torch.cuda.synchronize()
        ms = s.elapsed_time(e) / calls
    finally:
        settings.precision = old
    n = psi.size
    return {"workload": f"diagonal-Coulomb evolve t=0.1, norb={norb} ({na}a,{nb}b), "
                        f"{n} determinants, seed {SEED}",
            "ms": ms, "hbm_gbs": 32.0 * n / (ms / 1e3) / 1e9,
            "norm_after": float(torch.linalg.norm(w.get_coeff(key)))}


def rdm_leg(norb=14):
    """One- and two-particle RDMs (FqeData.rdm1 / rdm12) of the norb
    (norb/2, norb/2) sector's seeded wavefunction, CUDA events: rdm1 three
    times, rdm12 once after a warm-up, and rdm12's FP64 rate on the
    Hermitian half of its Gram matrix (norb^2 (norb^2 + 1) / 2 complex
    multiply-adds per determinant)."""
    import torch
    import fqe_gb300
    from fqe_gb300 import synthetic
    na = nb = norb // 2
    _, _, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), SEED)
    d = fqe_gb300.FqeData(na, nb, norb)
    d.set_wfn(strategy="from_data", raw_data=psi)

    def timed(fn, reps=1):
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            fn()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / reps

    d.rdm1()
    t1 = timed(lambda: d.rdm1(), 3)
    d.rdm12()
    t12 = timed(lambda: d.rdm12())
    p, n = norb * norb, psi.size
    return {"workload": f"rdm1 and rdm12, norb={norb} ({na}a,{nb}b), {n} determinants",
            "rdm1_ms": t1, "rdm12_ms": t12,
            "rdm12_fp64_tflops": 8.0 * p * (p + 1) / 2 * n / (t12 / 1e3) / 1e12}


def rows_leg():
    """The rows either side of the apply, timed once each after a warm-up
    (CUDA events / wall clock): the spin-orbital two-body apply
    (FqeData.apply with 2 norb spin orbitals) at norb 12 (6a,6b) on the
    tensor cores and in FP64, with their relative difference; the orbital
    rotation Wavefunction.transform of the norb-14 (7a,7b) sector under a
    seeded random unitary (2 norb column passes); and save + read of that
    wavefunction through a temporary file."""
    import numpy
    import torch
    import fqe_gb300
    from fqe_gb300 import settings, synthetic

    def timed(fn):
        torch.cuda.synchronize()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        r = fn()
        e.record()
        torch.cuda.synchronize()
        return r, s.elapsed_time(e)

    out = {}
    old = settings.precision
    try:
        norb, na, nb = 12, 6, 6
        rng = numpy.random.default_rng(SEED + 12)
        h1s, h2s, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), SEED)
        # spin-orbital integrals: the spatial ones in both spin blocks plus an
        # alpha-beta asymmetry, so the operator is not spin-free
        n2 = 2 * norb
        h1 = numpy.zeros((n2, n2))
        h1[:norb, :norb] = h1s
        h1[norb:, norb:] = h1s + 0.01 * numpy.diag(rng.normal(size=norb))
        h2 = numpy.zeros((n2,) * 4)
        for sa in (0, norb):
            for sb in (0, norb):
                h2[sa:sa + norb, sb:sb + norb, sa:sa + norb, sb:sb + norb] = h2s
        d = fqe_gb300.FqeData(na, nb, norb)
        d.set_wfn(strategy="from_data", raw_data=psi)
        res = {}
        row = {}
        for prec in ("ozaki", "fp64"):
            settings.precision = prec
            d.apply((h1, h2))
            r, ms = timed(lambda: d.apply((h1, h2)))
            res[prec] = r.coeff.clone()
            row[f"{prec}_ms"] = ms
        row["rel_diff_ozaki_vs_fp64"] = float(torch.linalg.norm(res["ozaki"] - res["fp64"])
                                              / torch.linalg.norm(res["fp64"]))
        row["workload"] = (f"spin-orbital apply, norb={norb} ({na}a,{nb}b), "
                           f"{psi.size} determinants, {2 * norb} spin orbitals")
        out["spin_orbital_apply"] = row
        del res, d
        settings.precision = "fp64"
        norb, na, nb = 14, 7, 7
        key = (na + nb, 0)
        _, _, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), SEED)
        w = fqe_gb300.Wavefunction([[na + nb, 0, norb]])
        w.set_wfn(strategy="from_data", raw_data={key: psi})
        a = rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb))
        u, _ = numpy.linalg.qr(a)
        w.transform(u)
        _, ms = timed(lambda: w.transform(u))
        out["orbital_rotation"] = {
            "workload": f"Wavefunction.transform, norb={norb} ({na}a,{nb}b), "
                        f"{psi.size} determinants, random unitary",
            "ms": ms, "norm_after": float(torch.linalg.norm(w.get_coeff(key)))}
        with tempfile.TemporaryDirectory() as tmp:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            w.save("wfn.pkl", tmp)
            t1 = time.perf_counter()
            w2 = fqe_gb300.Wavefunction([[na + nb, 0, norb]])
            w2.read("wfn.pkl", tmp)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            same = bool(torch.equal(w2.get_coeff(key), w.get_coeff(key)))
        out["save_read"] = {"workload": f"save + read, norb={norb}, {psi.size * 16} bytes",
                            "save_s": t1 - t0, "read_s": t2 - t1, "identical": same}
    finally:
        settings.precision = old
    return out


def taylor_leg(norb=16, steps=20, dt=0.05, accuracy=1e-12, fp64_check=True):
    """The norb-16 (8a,8b) configuration: `steps` Taylor steps of dt on the
    tensor cores (Ozaki-split BF16), per step the wall time, the number of
    terms, the norm and the energy <psi|H|psi>; the first step also on the
    FP64 GPU path, with the relative difference and the fidelity
    |<psi_oz|psi_fp64>|^2 of the two results."""
    import torch
    import fqe_gb300
    from fqe_gb300 import settings, synthetic
    na, nb = norb // 2, norb - norb // 2
    nchol = synthetic.default_nchol(norb)
    h1, h2, psi = synthetic.sector(norb, na, nb, nchol, SEED)
    ham = fqe_gb300.RestrictedHamiltonian((h1, h2))
    key = (na + nb, na - nb)
    w0 = fqe_gb300.Wavefunction([[na + nb, na - nb, norb]])
    w0.set_wfn(strategy="from_data", raw_data={key: psi})
    del psi
    old = settings.precision
    out = {"workload": f"norb={norb} ({na}a,{nb}b), {nchol} Cholesky vectors, seed {SEED}; "
                       f"{steps} Taylor steps dt={dt} to {accuracy}"}
    try:
        settings.precision = "ozaki"
        w = w0
        rows = []
        for k in range(steps):
            torch.cuda.synchronize()
            t0 = time.time()
            w = w.apply_generated_unitary(dt, "taylor", ham, accuracy=accuracy,
                                          expansion=80)
            torch.cuda.synchronize()
            sec = time.time() - t0
            if k == 0:
                first = w.get_coeff(key).clone()
            e = complex(w.expectationValue(ham))
            rows.append({"step": k + 1, "seconds": sec, "terms": w._taylor_terms,
                         "norm_minus_1": w.norm() - 1.0, "energy": e.real,
                         "energy_imag": e.imag})
        out["ozaki_steps"] = rows
        out["norm_drift_max"] = max(abs(r["norm_minus_1"]) for r in rows)
        out["energy_drift_max"] = max(abs(r["energy"] - rows[0]["energy"]) for r in rows)
        if fp64_check:
            settings.precision = "fp64"
            torch.cuda.synchronize()
            t0 = time.time()
            w64 = w0.apply_generated_unitary(dt, "taylor", ham, accuracy=accuracy,
                                             expansion=80)
            torch.cuda.synchronize()
            ref = w64.get_coeff(key)
            out["fp64_first_step_seconds"] = time.time() - t0
            out["first_step_rel_diff_vs_fp64"] = float(
                torch.linalg.norm(first - ref) / torch.linalg.norm(ref))
            ov = torch.vdot(first.reshape(-1), ref.reshape(-1))
            out["first_step_infidelity_vs_fp64"] = float(
                1.0 - abs(ov) ** 2 / (torch.linalg.norm(first) ** 2 *
                                      torch.linalg.norm(ref) ** 2))
    finally:
        settings.precision = old
    return out


BATCH_SHAPES = {8: [(4, 4), (5, 3), (3, 5), (4, 3), (5, 4)],
                10: [(5, 5), (6, 4), (4, 5), (5, 4)],
                12: [(6, 6), (5, 6), (6, 5), (7, 5)]}


def batch_sectors(n=256):
    """The batched configuration: n wavefunctions over norb {8, 10, 12} with
    uneven (nalpha, nbeta), each with its own seeded integrals (seed = index)
    and random normalised psi."""
    from fqe_gb300 import synthetic
    out = []
    for i in range(n):
        norb = (8, 10, 12)[i % 3]
        shapes = BATCH_SHAPES[norb]
        na, nb = shapes[(i // 3) % len(shapes)]
        h1, h2, psi = synthetic.sector(norb, na, nb, synthetic.default_nchol(norb), i)
        out.append((norb, na, nb, h1, h2, psi))
    return out


def batch_leg(n=256, reps=5):
    """Benchmark configuration 3 on the tensor-core precision: n uneven
    sectors' applies in one CUDA graph (fqegpu_batch_*) and their Taylor
    evolutions t = 0.1 to 1e-10 in one graph (fqegpu_batch_taylor_*), with the
    default launch shape ("fixed") and with the autotuner's per-shape choice
    ("autotuned"); CUDA events around the graph launches."""
    import gc
    import torch
    import fqe_gb300
    from fqe_gb300 import autotune, settings
    from fqe_gb300.batch import BatchApply, BatchTaylor
    secs = batch_sectors(n)
    ndet = sum(p[5].size for p in secs)
    out = {"workload": f"{n} sectors, norb {{8,10,12}} uneven (nalpha, nbeta), "
                       f"{ndet} determinants in all; apply + Taylor t=0.1 to 1e-10",
           "determinants": ndet}

    def datas():
        ds = []
        for norb, na, nb, h1, h2, psi in secs:
            d = fqe_gb300.FqeData(na, nb, norb)
            d.set_wfn(strategy="from_data", raw_data=psi)
            ds.append(d)
        return ds

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    arrays = [(p[3], p[4]) for p in secs]
    old = settings.precision
    settings.precision = "ozaki"
    try:
        for tuned in (False, True):
            tag = "autotuned" if tuned else "fixed"
            autotune.clear()
            ds = datas()
            b = BatchApply(ds, arrays, precision="ozaki", autotune=tuned)
            b.launch()
            b.check()
            ms = min(timed(lambda: (b.launch(), b.check())) for _ in range(reps))
            choices = {}
            if tuned:
                for k, v in autotune.cached().items():
                    choices[f"{k[0]}_{k[1]}_{k[2]}"] = (
                        "fp64" if v["fp64"] else f"tensor/super{v['super_tiles']}")
            out[f"apply_{tag}"] = {"ms": ms, "det_per_s": ndet / (ms / 1e3)}
            if tuned:
                out["autotuned_choices"] = choices
            del b
            gc.collect()
            ds = datas()
            bt = BatchTaylor(ds, arrays, 0.1, accuracy=1e-10, expansion=80,
                             precision="ozaki", autotune=tuned)
            ms_t = timed(lambda: (bt.launch(), bt.terms()))
            terms = bt.terms()
            out[f"taylor_{tag}"] = {"ms": ms_t, "terms_min": min(terms),
                                    "terms_max": max(terms)}
            del bt, ds
            gc.collect()
            torch.cuda.empty_cache()
    finally:
        settings.precision = old
    return out


def _block_w(ham):
    import numpy
    from fqe_gb300 import _lib
    info = numpy.zeros(4, dtype=numpy.int64)
    _lib.call("fqegpu_ham_info", ham.handle, info.ctypes.data_as(ctypes.c_void_p))
    lena = math.comb(NORB, NALPHA)
    per_col = 2 * info[0] * lena * 16
    return int(info[3] // per_col) if info[3] else math.comb(NORB, NBETA)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--precision", choices=["auto", "fp64", "ozaki"],
                    default="auto")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--norb", type=int, default=14)
    ap.add_argument("--nalpha", type=int, default=None)
    ap.add_argument("--nbeta", type=int, default=None)
    ap.add_argument("--nchol", type=int, default=None)
    ap.add_argument("--no-davidson", action="store_true",
                    help="skip the Davidson (plain vs learned) leg")
    ap.add_argument("--davidson-norb", type=int, default=12)
    ap.add_argument("--davidson-subspace", type=int, default=32)
    ap.add_argument("--davidson-scratch-gb", type=float, default=None,
                    help="device workspace of the Davidson applies (GB)")
    ap.add_argument("--davidson-max-iter", type=int, default=400)
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="with --taylor16: skip the first step's FP64 comparison")
    ap.add_argument("--batch", action="store_true",
                    help="only the batched configuration: 256 uneven sectors, "
                         "apply and Taylor graphs, fixed vs autotuned")
    ap.add_argument("--taylor16", action="store_true",
                    help="only the norb-16 (8a,8b) 20-step Taylor evolution "
                         "(tensor cores) with the first step against FP64")
    ap.add_argument("--rows", action="store_true",
                    help="only the rows beside the apply: spin-orbital apply, "
                         "orbital rotation, save/read")
    ap.add_argument("--rdm", action="store_true",
                    help="only the norb-14 one- and two-particle RDMs")
    ap.add_argument("--diag", action="store_true",
                    help="only the norb-14 diagonal-Coulomb evolve (20 timed calls)")
    ap.add_argument("--configs", action="store_true",
                    help="only measure the other single-GPU configurations "
                         "(norb 8 apply/Taylor; norb 14 FP64 vs tensor-core "
                         "error, Taylor, diagonal-Coulomb evolve)")
    args = ap.parse_args()
    if args.norb != 14 or args.nalpha is not None or args.nbeta is not None:
        na = args.nalpha if args.nalpha is not None else args.norb // 2
        nb = args.nbeta if args.nbeta is not None else args.norb - args.norb // 2
        from fqe_gb300 import synthetic
        set_workload(args.norb, na, nb,
                     args.nchol or synthetic.default_nchol(args.norb))
    if args.impl == "reference":
        return run_reference(args)
    if args.configs or args.taylor16 or args.batch or args.diag or args.rdm or args.rows:
        import torch
        import fqe_gb300
        torch.cuda.set_device(0)
        fqe_gb300.build()
        if args.batch:
            print(json.dumps({"batch": batch_leg()}), flush=True)
        elif args.diag:
            print(json.dumps({"diag_coulomb": diag_leg()}), flush=True)
        elif args.rdm:
            print(json.dumps({"rdm": rdm_leg()}), flush=True)
        elif args.rows:
            print(json.dumps({"rows": rows_leg()}), flush=True)
        elif args.taylor16:
            print(json.dumps({"taylor_norb16": taylor_leg(
                fp64_check=not args.no_fp64_check)}), flush=True)
        else:
            print(json.dumps({"configs": configs_leg()}), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
