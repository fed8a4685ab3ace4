"""Benchmark of the H.X hot kernel on the standalone lattice workload.

Workload: 40^3 lattice, h = 0.5 fm, a block of 64 complex 2-spinors with
seeded Gaussian components orthonormalised in FP64, seeded U / f / W fields
(nuclearcgm_gb300.workloads). One step = one H.X over the whole block.
Metric: H.X throughput in GB/s of algorithmic bytes, where the bytes of one
H.X are those of the FP32 workload: X read once + Y written once + the 8
per-point field values, 133.1 MB (the same unit for every arm, so the ratio
of two lines is the ratio of their times per H.X).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Our arm times the FP32 TMA stencil on device-resident inputs with CUDA events
on the launching stream; inputs rotate over 4 block pairs (524 MB > 129 MB
L2) so every step reads from HBM. `e2e` is the same metric through the
reference-facing C-ABI call ncgm_apply_h with pinned HOST buffers in the
Eigen layout (complex<double>), copies included. The reference arm times the
CPU restatement of the reference's assembled-CSR product (FP64) on all host
cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

N_LAT, H_LAT, NCOLS = 40, 0.5, 64
METRIC = "H.X HBM GB/s (algorithmic bytes) on 40^3 x 64 spinors"


def _peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(0.25)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def _workload():
    from nuclearcgm_gb300 import workloads
    a, f, gradf, U, W = workloads.fields(N_LAT, H_LAT)
    X = workloads.orthonormal_block(2 * N_LAT ** 3, NCOLS, seed=1)
    return a, f, gradf, U, W, X


def _cpu_reference(steps, warmup, a, f, gradf, U, W, X, cols_per_step):
    """Times the FP64 CSR product of the oracle (the reference's assembled
    Hamiltonian times a dense block) on all host threads."""
    import numpy as np
    from nuclearcgm_gb300 import workloads
    from oracle import oracle
    H = oracle.Hamiltonian.skyrme(N_LAT, a, f, gradf.T, U, W.T)
    Xs = np.asfortranarray(X[:, :cols_per_step])
    for _ in range(warmup):
        H.apply(Xs)
    t0 = time.perf_counter()
    for _ in range(steps):
        H.apply(Xs)
    dt = (time.perf_counter() - t0) / steps
    # throughput in the workload's unit: FP32-workload bytes of the columns
    # processed per step
    byts = workloads.hx_bytes(N_LAT, cols_per_step, 4)
    return byts / dt / 1e9, dt


O16_HF = {"functional": "SLy4", "nucleus": {"A": 16, "Z": 8},
          "box": {"boxSize": 18.0, "axisMeshPoints": 30},
          "maxIterations": 500, "energyTol": 1e-3}


CA40_HF = {"functional": "SLy4", "nucleus": {"A": 40, "Z": 20},
           "box": {"boxSize": 20.0, "axisMeshPoints": 36},
           "maxIterations": 500, "energyTol": 1e-3}


def _hf_wall_ca40():
    """The learned-preconditioner evaluation nucleus: 40Ca, SLy4, 36^3
    lattice, box 20 fm, 20 orbitals per isospin, to |dE| < 1 keV, in the
    plain FP64, mixed, mixed + tensor-core and learned + mixed forms (second
    of two runs each)."""
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi, config
    lp = None
    wpath = os.path.join(HERE, "nuclearcgm_gb300", "data", "lp_weights.f32")
    if os.path.exists(wpath):
        lp = ng.LearnedPreconditioner.pretrained(wpath)
    out = {"workload": "40Ca HF ground state, SLy4, 36^3 lattice, box 20 fm, "
                       "|dE| < 1 keV", "unit": "s"}
    forms = [("fp64_gpu", abi.FP64, abi.PRECOND_JACOBI),
             ("mixed_gpu", abi.FP32, abi.PRECOND_JACOBI),
             ("mixed_tc_gpu", abi.FP32_TC, abi.PRECOND_JACOBI)]
    if lp is not None:
        forms.append(("learned_mixed_gpu", abi.FP32, abi.PRECOND_LEARNED))
        forms.append(("learned_mixed_tc_gpu", abi.FP32_TC,
                      abi.PRECOND_LEARNED))
    for name, prec, pc in forms:
        cfg = config.from_input(CA40_HF, precision=prec)
        cfg.hf_gcg.precond = pc
        if pc == abi.PRECOND_LEARNED:
            cfg.lp = lp.h.value
        for rep in range(2):
            t0 = time.perf_counter()
            res, _ = ng.hf_run(cfg)
            wall = time.perf_counter() - t0
        out[name + "_s"] = round(wall, 4)
        out[name + "_iterations"] = res.iterations
        out[name + "_E_MeV"] = round(res.E_HF, 6)
        out[name + "_gcg_s"] = round(res.t_gcg_s, 4)
    return out


SN120_HFB = {"functional": "SLy4", "nucleus": {"A": 120, "Z": 50},
             "box": {"boxSize": 24.0, "axisMeshPoints": 48},
             "pairing": {"type": "HFB", "HFbasisSize": 160, "V0": 300.0,
                         "window": 60.0},
             "maxIterations": 400, "energyTol": 1e-3}


def _hf_wall_sn120(forms=("mixed_tc_gpu", "fp64_gpu")):
    """120Sn HFB ground state: SLy4, 48^3 lattice, box 24 fm, 160
    quasiparticle states per isospin, zero-range pairing V0 = 300 with a
    60 MeV window, Coulomb by the Poisson solve, to |dE| < 1 keV (one run
    per form; minutes each, so only with --sn120)."""
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi, config
    out = {"workload": "120Sn HFB ground state, SLy4, 48^3 lattice, box "
                       "24 fm, 160 states per isospin, V0 300, 60 MeV "
                       "window, |dE| < 1 keV", "unit": "s"}
    precs = {"fp64_gpu": abi.FP64, "mixed_tc_gpu": abi.FP32_TC}
    for name in forms:
        cfg = config.from_input(SN120_HFB, precision=precs[name])
        t0 = time.perf_counter()
        res, _ = ng.hf_run(cfg)
        out[name + "_s"] = round(time.perf_counter() - t0, 3)
        out[name + "_iterations"] = res.iterations
        out[name + "_converged"] = bool(res.converged)
        out[name + "_E_MeV"] = round(res.E_HF, 6)
        out[name + "_E_int_MeV"] = round(res.E_int, 6)
        out[name + "_E_pair_n_MeV"] = round(res.E_pair_n, 6)
        out[name + "_E_pair_p_MeV"] = round(res.E_pair_p, 6)
        out[name + "_phase_s"] = {"gcg": round(res.t_gcg_s, 3),
                                  "fields": round(res.t_fields_s, 3),
                                  "poisson": round(res.t_poisson_s, 3),
                                  "pairing": round(res.t_pairing_s, 3)}
    return out


def _curve_cfg2():
    """The 24Mg deformation curve: SkM*, 32^3 lattice, box 20 fm, HF+BCS
    with 24 states per isospin, 16 beta2 points in [-0.3, 0.5] under the
    curve-mode constraint set (main.cpp:176-185), each to |dE| < 1 keV.
    Timed: all 16 points at once (ncgm_hf_run_batch, one stream and
    context per point) in the FP64 and tensor-core forms, and the points one
    after the other in the tensor-core form; per-point |dE| of the
    tensor-core form against its own FP64 run. The CPU leg is the oracle's
    measured cost per HF iteration at this size (tests/golden fixture
    generation on the development host) times the FP64 iteration counts."""
    import numpy as np
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi
    sys.path.insert(0, os.path.join(HERE, "tests", "golden"))
    import make_fixtures as mf
    out = {"workload": "24Mg HF+BCS curve, SkM*, 32^3 lattice, box 20 fm, "
                       "24 states per isospin, 16 beta2 points in "
                       "[-0.3, 0.5], |dE| < 1 keV per point", "unit": "s"}
    res = {}
    for name, prec in (("fp64", abi.FP64), ("tc", abi.FP32_TC)):
        cfgs = mf.curve_configs(mf.MG24, prec, 1e-3, 500)
        t0 = time.perf_counter()
        res[name] = ng.hf_run_batch(cfgs)
        out["batched_%s_s" % name] = round(time.perf_counter() - t0, 3)
    cfgs = mf.curve_configs(mf.MG24, abi.FP32_TC, 1e-3, 500)
    t0 = time.perf_counter()
    for c in cfgs:
        ng.hf_run(c)
    out["serial_tc_s"] = round(time.perf_counter() - t0, 3)
    e64 = np.array([r.E_HF for r in res["fp64"]])
    etc = np.array([r.E_HF for r in res["tc"]])
    out["E_HF_fp64_MeV"] = [round(x, 6) for x in e64]
    out["beta_fp64"] = [round(r.beta, 5) for r in res["fp64"]]
    out["iterations_fp64"] = [r.iterations for r in res["fp64"]]
    out["converged"] = [bool(r.converged) for r in res["fp64"]]
    out["abs_dE_tc_vs_fp64_MeV"] = [float("%.3g" % x)
                                    for x in np.abs(etc - e64)]
    out["max_abs_dE_tc_vs_fp64_MeV"] = float(np.abs(etc - e64).max())
    out["iterations_tc"] = [r.iterations for r in res["tc"]]
    out["converged_tc"] = [bool(r.converged) for r in res["tc"]]
    # the oracle's measured seconds per HF iteration at this size
    per_it = []
    for name in ("mg24_skm_n32_p00", "mg24_skm_n32_p07", "mg24_skm_n32_p15"):
        if os.path.exists(mf.path(name)):
            fx = mf.load(name)
            per_it.append(float(fx["oracle_seconds"]) /
                          int(fx["iterations"]))
    if per_it:
        s_it = float(np.mean(per_it))
        out["cpu_oracle_s_per_iteration"] = round(s_it, 3)
        out["cpu_oracle_s_est"] = round(
            s_it * sum(r.iterations for r in res["fp64"]), 1)
        out["cpu_note"] = ("oracle FP64 seconds per iteration measured while "
                           "generating the 24Mg fixtures (x86 host, all "
                           "cores) times the 16 points' FP64 GPU iteration "
                           "counts")
    return out


def _hf_wall(with_cpu):
    """Wall seconds to |dE| < 1 keV (the driver's stop rule, main.cpp:333-337)
    for the 16O HF ground state (SLy4, 30^3 lattice, box 18 fm, Woods-Saxon
    guess) in three device forms: plain FP64, mixed (FP32 PCG corrections),
    and learned + mixed (PCG started from the trained network). Each form
    runs twice in this process and the second run is timed (the first pays
    the one-off stencil autotuning and allocations)."""
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi, config
    lp = None
    wpath = os.path.join(HERE, "nuclearcgm_gb300", "data", "lp_weights.f32")
    if os.path.exists(wpath):
        lp = ng.LearnedPreconditioner.pretrained(wpath)
    forms = [("fp64_gpu", abi.FP64, abi.PRECOND_JACOBI),
             ("mixed_gpu", abi.FP32, abi.PRECOND_JACOBI),
             ("mixed_tc_gpu", abi.FP32_TC, abi.PRECOND_JACOBI)]
    if lp is not None:
        forms.append(("learned_mixed_gpu", abi.FP32, abi.PRECOND_LEARNED))
        forms.append(("learned_mixed_tc_gpu", abi.FP32_TC,
                      abi.PRECOND_LEARNED))
    out = {"workload": "16O HF ground state, SLy4, 30^3 lattice, box 18 fm, "
                       "|dE| < 1 keV", "unit": "s"}
    for name, prec, pc in forms:
        cfg = config.from_input(O16_HF, precision=prec)
        cfg.hf_gcg.precond = pc
        if pc == abi.PRECOND_LEARNED:
            cfg.lp = lp.h.value
        for rep in range(2):
            t0 = time.perf_counter()
            res, _ = ng.hf_run(cfg)
            wall = time.perf_counter() - t0
        out[name + "_s"] = round(wall, 4)
        out[name + "_iterations"] = res.iterations
        out[name + "_E_MeV"] = round(res.E_HF, 6)
    if lp is None:
        out["learned_mixed_gpu_s"] = None
        out["learned_note"] = "no trained weights (nuclearcgm_gb300.train_lp)"
    if with_cpu:
        # the FP64 CPU oracle on the same input to the same stop rule, timed
        from oracle import oracle
        c = config.from_input(O16_HF)
        t0 = time.perf_counter()
        ro, _ = oracle.hf_run(c)
        out["cpu_oracle_s"] = round(time.perf_counter() - t0, 3)
        out["cpu_oracle_iterations"] = ro.iterations
        out["cpu_oracle_E_MeV"] = round(ro.E_HF, 6)
        out["cpu_cores"] = os.cpu_count()
    return out


def _gcg_step(H, X):
    """One GCG iteration (reference parameters: 80 PCG steps, cgTol 1e-5) on
    the 40^3 x 64 workload in the plain FP64 form, the FP32-correction form
    and the FP32 + tensor-core Gram form, from a block first brought near
    the eigenpairs (12 FP64 iterations from the seeded orthonormal block);
    eigenvalue differences against the FP64 step."""
    from nuclearcgm_gb300 import abi
    out = {"workload": "one GCG iteration, 40^3 lattice, 64 spinors, "
                       "80 PCG steps max, cgTol 1e-5, from 12 FP64 "
                       "iterations of the seeded block", "unit": "ms"}
    warm = abi.GcgParams(max_iter=12, tol=1e-6, cg_steps=80, cg_tol=1e-5,
                         shift=0, ordering=1, precision=abi.FP64, precond=0)
    X = H.gcg(X, 64, None, warm)[0]
    lam = {}
    for name, prec in (("fp64", abi.FP64), ("fp32", abi.FP32),
                       ("fp32_tc", abi.FP32_TC)):
        p = abi.GcgParams(max_iter=1, tol=1e-6, cg_steps=80, cg_tol=1e-5,
                          shift=0, ordering=1, precision=prec, precond=0)
        H.gcg(X, 64, None, p)
        t = []
        for _ in range(3):
            _, lam[name], st = H.gcg(X, 64, None, p)
            t.append(st.ms_total)
        out[name + "_ms"] = round(min(t), 3)
        out[name + "_pcg_ms"] = round(st.ms_pcg, 3)
    import numpy as np
    for name in ("fp32", "fp32_tc"):
        d = np.abs(lam[name] - lam["fp64"])
        out[name + "_max_dlambda_MeV"] = float(d.max())
        # the lowest half of the block (converged furthest) separately
        out[name + "_max_dlambda_low32_MeV"] = float(d[:32].max())
    return out


# FP64 pipe instructions of the operator per point and column, counted from
# its arithmetic (stencil_core.cuh pointH): 65 additions, 8 multiplications
# and 56 FMAs (185 flops)
FP64_OPS_PER_POINT_COL = 129
FP64_FLOPS_PER_POINT_COL = 185


def _fp64_roofline(lib, ms64):
    """The FP64 stencil against the FP64 pipe: pipe instructions per second
    of the apply over FMA instructions per second of the probe kernel
    (ncgm_measure_fp64_gflops / 2); an addition or a multiplication takes a
    pipe slot like an FMA."""
    import ctypes
    from nuclearcgm_gb300 import workloads
    pts = N_LAT ** 3 * NCOLS
    out = {"ms_per_hx": round(ms64, 4),
           "gbs": round(workloads.hx_bytes(N_LAT, NCOLS, 8) /
                        (ms64 * 1e-3) / 1e9, 2),
           "gflops": round(pts * FP64_FLOPS_PER_POINT_COL / (ms64 * 1e-3) /
                           1e9, 1)}
    g = ctypes.c_double(0)
    if lib.ncgm_measure_fp64_gflops(ctypes.byref(g)) == 0 and g.value > 0:
        ops = pts * FP64_OPS_PER_POINT_COL / (ms64 * 1e-3) / 1e9
        out["roofline"] = {"bound": "fp64 pipe", "achieved": round(ops, 1),
                           "peak": round(g.value / 2, 1),
                           "unit": "G FP64 instructions/s",
                           "frac": round(ops / (g.value / 2), 4),
                           "peak_source": "measured (ncgm_measure_fp64_"
                                          "gflops: %.1f GFLOP/s)" % g.value}
    return out


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    a, f, gradf, U, W, X = _workload()
    cores = os.cpu_count()
    gbs, dt = _cpu_reference(args.steps, min(args.warmup, 2), a, f, gradf, U,
                             W, X, NCOLS)
    line = {
        "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "H.X 40^3 lattice, 64 complex 2-spinors, "
                               "h=0.5 fm",
                   "global_batch": NCOLS, "seq_len": 2 * N_LAT ** 3,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s",
                         "cores": cores, "kind": "port",
                         "sample": "the whole 64-column block per step (FP64 "
                                   "CSR product), CSR assembled once (not "
                                   "timed)"},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    import nuclearcgm_gb300 as ng
    from nuclearcgm_gb300 import abi, workloads

    ws, rank = _dist()
    if ws > 1:
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    a, f, gradf, U, W, X = _workload()
    grid = ng.Grid(N_LAT, a)
    ctx = ng.Context(grid, NCOLS)
    H = ng.Hamiltonian(ctx, abi.NEUTRON).set_fields(f, gradf.T, U, W.T)
    lib = ng.load()
    # a dedicated (non-default) stream: kernels and CUDA events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ng._check(lib.ncgm_set_stream(ctx.h, stream.cuda_stream))
    Nrow = 2 * N_LAT ** 3
    xt = torch.from_numpy(np.ascontiguousarray(X.T)).to(torch.complex64)
    sets = 4  # 4 x (X + Y) x 65.5 MB = 524 MB > 129 MB L2
    Xs = [xt.cuda() for _ in range(sets)]
    Ys = [torch.empty_like(Xs[0]) for _ in range(sets)]
    tune = lib.ncgm_apply_h_device

    def step(i):
        ng._check(tune(ctx.h, 0, Xs[i % sets].data_ptr(),
                       Ys[i % sets].data_ptr(), NCOLS, abi.FP32, 0.0))

    for i in range(max(args.warmup, 3)):
        step(i)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(args.steps):
            step(i)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    ms_step = ms / args.steps
    byts = workloads.hx_bytes(N_LAT, NCOLS, 4)
    value = byts * ws / (ms_step * 1e-3) / 1e9
    # parity spot check of this exact workload against FP64 (not timed)
    Y32 = Ys[0].cpu().numpy().T.astype(np.complex128)
    Y64 = H.apply(X)
    rel32 = float(np.abs(Y32 - Y64).max() / np.abs(Y64).max())

    # FP64 stencil, same workload (device-resident), for the record
    x64 = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    y64 = torch.empty_like(x64)
    for _ in range(3):
        ng._check(tune(ctx.h, 0, x64.data_ptr(), y64.data_ptr(), NCOLS,
                       abi.FP64, 0.0))
    torch.cuda.synchronize()
    e0.record(stream)
    r64 = 10
    for _ in range(r64):
        ng._check(tune(ctx.h, 0, x64.data_ptr(), y64.data_ptr(), NCOLS,
                       abi.FP64, 0.0))
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / r64

    # e2e through the C-ABI with pinned host buffers (copies timed)
    ng._check(lib.ncgm_set_stream(ctx.h, None))
    xh = torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    ke = max(3, min(args.steps, 20))
    ng._check(lib.ncgm_apply_h(ctx.h, 0, xh.data_ptr(), yh.data_ptr(), NCOLS,
                               abi.FP32))
    t0 = time.perf_counter()
    for _ in range(ke):
        ng._check(lib.ncgm_apply_h(ctx.h, 0, xh.data_ptr(), yh.data_ptr(),
                                   NCOLS, abi.FP32))
    te = (time.perf_counter() - t0) / ke
    e2e = byts / te / 1e9
    h2d = Nrow * NCOLS * 16

    peak, peak_kind = _peaks()
    traffic = None
    tp = os.path.join(HERE, "profiles", "stencil_fp32_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    hf = gstep = hf_ca = curve = None
    if rank == 0 and not args.no_hf:
        gstep = _gcg_step(H, X)
        hf = _hf_wall(not args.no_cpu)
        hf_ca = _hf_wall_ca40()
    curve = _curve_cfg2() if (rank == 0 and args.curve) else None
    sn = _hf_wall_sn120() if (rank == 0 and args.sn120) else None
    cpu = None
    if rank == 0 and not args.no_cpu:
        gbs_c, dt_c = _cpu_reference(3, 1, a, f, gradf, U, W, X, NCOLS)
        cpu = {"value": round(gbs_c, 3), "unit": "GB/s",
               "cores": os.cpu_count(), "kind": "port",
               "sample": "the whole 64-column block, 3 timed products "
                         "(FP64 CSR)"}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded splitmix64 fields and spinors)",
        "config": {"workload": "H.X 40^3 lattice, 64 complex 2-spinors, "
                               "h=0.5 fm, FP32 TMA stencil",
                   "global_batch": NCOLS * ws, "seq_len": Nrow,
                   "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "4 rotating X/Y sets (524 MB > 129 MB L2)"},
        "roofline": {"bound": "hbm", "achieved": round(byts / (ms_step * 1e-3)
                                                       / 1e9, 2),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(byts / (ms_step * 1e-3) / 1e9 / peak, 4),
                     "traffic": traffic, "peak_source": peak_kind},
        "e2e": {"value": round(e2e, 3), "unit": "GB/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
        "fp32_rel_err_vs_fp64": rel32,
        "fp64_stencil": _fp64_roofline(lib, ms64),
        "cpu_baseline": cpu,
        "hf_wall_to_1keV": hf,
        "hf_wall_to_1keV_ca40": hf_ca,
        "curve_cfg2": curve,
        "hf_wall_to_1keV_sn120": sn,
        "gcg_step": gstep,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU-baseline sample on our arm")
    ap.add_argument("--curve", action="store_true",
                    help="also time the 16-point 24Mg curve (about 8 minutes)")
    ap.add_argument("--sn120", action="store_true",
                    help="also time the 120Sn HFB run to 1 keV (minutes)")
    ap.add_argument("--no-hf", action="store_true",
                    help="skip the HF wall-time-to-convergence record")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
