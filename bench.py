#!/usr/bin/env python
"""SCF iterations/s of the bulk AB-diblock SCF loop on one GB300.

Workload: 128^3 grid, Ns = 200 (ds = 0.005, N_A = 80, N_B = 120), f_A = 0.40,
chi N = 20, kappa = 25, cubic box L = 3.8 R_g, canonical ensemble, Anderson
mixing with history m = 10 (lambda = 0.1).  Fields: the single-harmonic sum
of the 24 {211} plane waves with amplitude 0.5 plus seeded N(0, 0.05^2)
noise (synthetic, numpy default_rng).  A step is one whole SCF iteration
(both chains over all contour steps, contour integral, Q, mean fields,
residual, Anderson solve and mix), replayed from a CUDA graph.  The working
set (3.2 GB of FP32 propagator slices) is far larger than L2.

``python bench.py [--gpus N --steps K --warmup W]`` prints one JSON line.
``--impl reference`` times the CPU restatement of the reference instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("SCF iter/s @128^3,Ns=200: FP32/FP64-split vs FP64 GPU at "
          "|ΔF|≤1e-7; %HBM peak")
GRID = 128
L = 3.8
DS = 0.005
F_A = 0.40
CHI = 20.0
KAPPA = 25.0
M_HIST = 10
LAM = 0.1
SEED = 3
# DRAM bytes of one 128^3 FP32 double step (Yf, Z, Yi, X launches), measured with
# ncu on GB300: 17.53 MB, against 50.3 MB of algorithmic bytes (24 B per point)
DSTEP_TRAFFIC = 17_531_648
# L2 traffic of one 128^3 double step from the SM side, measured with ncu
# (lts__t_sectors_srcunit_tex.sum x 32 B of one launch each of the fused XY
# plane pass, 2,754,213 sectors, and of the TMA Z pass, 1,190,085 sectors;
# profiles/k_xy_tma_k_rs_tma_128cube_full.txt)
DSTEP_L2_BYTES = (2_754_213 + 1_190_085) * 32


def c3_fields(n=GRID, length=L, seed=SEED):
    """w_A = 0.5 S + noise, w_B = -0.5 S + noise; S = mean over the 12 +-pairs
    of {211} of cos(2 pi G.r / L); noise N(0, 0.05^2) per point and species."""
    rng = np.random.default_rng(seed)
    r = np.arange(n) * length / n
    z, y, x = np.meshgrid(r, r, r, indexing="ij")
    gs = set()
    import itertools
    for perm in set(itertools.permutations((2, 1, 1))):
        for sg in itertools.product((1, -1), repeat=3):
            g = tuple(p * s for p, s in zip(perm, sg))
            if tuple(-c for c in g) not in gs:
                gs.add(g)
    assert len(gs) == 12
    S = np.zeros((n, n, n))
    for gx, gy, gz in sorted(gs):
        S += np.cos(2 * np.pi * (gx * x + gy * y + gz * z) / length)
    S /= 12.0
    w = np.empty((2, n, n, n))
    w[0] = 0.5 * S + rng.normal(0.0, 0.05, S.shape)
    w[1] = -0.5 * S + rng.normal(0.0, 0.05, S.shape)
    return w


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def make_ctx(A, prec, stream=None):
    c = A.Context(A.BULK, grid=(GRID, GRID, GRID), size=(L, L, L), ds=DS,
                  block_length=(F_A, 1.0 - F_A), ensemble=1, rho=1.0, kappa=KAPPA,
                  chi=CHI, precision=prec, mixing_type=A.MIX_ANDERSON,
                  mixing_dim=M_HIST, lam=LAM, lam_warm=LAM, warm_iters=M_HIST)
    if stream is not None:
        A._lib.check(c.lib, c.h, c.lib.adscf_set_stream(c.h, stream.cuda_stream))
    return c


def time_stage(torch, ctx, stream, stage, reps):
    lib = ctx.lib
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx._ck(lib.adscf_enqueue(ctx.h, stage, reps))
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


# --------------------------------------------------------------------------
# CPU legs: the C++17/OpenMP FP64 restatement of the reference's iteration
# (oracle/scf_cpu.cpp; gfortran and FFTW, which the reference needs, are on
# neither machine), timed over whole SCF iterations of the same workload
# --------------------------------------------------------------------------
def cpu_model():
    """CPU model string and logical core count of this host."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            for line in Path("/proc/cpuinfo").read_text().splitlines():
                if line.startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return model or "unknown", os.cpu_count() or 1


def cpu_context():
    from oracle import cbuild
    return cbuild.ScfCpu((GRID, GRID, GRID), (L, L, L), DS, F_A, KAPPA, CHI, m=M_HIST, lam=LAM,
                         lam_warm=LAM, warm_iters=M_HIST)


def cpu_iterations(c, n):
    """Seconds per whole SCF iteration over n iterations of context c."""
    t0 = time.perf_counter()
    c.iterate(n)
    return (time.perf_counter() - t0) / n


def config(world):
    return {"workload": "bulk diblock 128^3 Ns=200 f_A=0.40 chiN=20 kappa=25 L=3.8 "
                        "canonical, Anderson m=10, {211} fields + noise",
            "grid": [GRID, GRID, GRID], "ns": 200, "parallelism": f"replicas{world}",
            "l2": "working set 3.4 GB > L2 (no flush needed)"}


def run_reference(args):
    """Whole SCF iterations of the workload on all host cores: W untimed,
    then K timed, each a full iteration (both chains over 200 contour
    steps, contour integral, mean fields, Anderson mix)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import cbuild
    lib = cbuild.load()
    model, ncpu = cpu_model()
    threads = lib.scfcpu_threads()
    t_start = time.perf_counter()
    with cpu_context() as c:
        c.set_field(c3_fields())
        c.iterate(args.warmup)
        sec = cpu_iterations(c, args.steps)
    v = 1.0 / sec
    sample = (f"{args.steps} whole SCF iterations after {args.warmup} untimed, C++17/OpenMP FP64 "
              f"restatement of the reference (oracle/scf_cpu.cpp; its own FFT; gfortran/FFTW "
              f"absent), {threads} threads on {ncpu} logical cores, {model}")
    out = {
        "metric": METRIC, "value": v, "unit": "iter/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sec, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(args.gpus),
        "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": sample, "cpu_model": model, "nproc": ncpu},
        "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.perf_counter() - t_start,
    }
    print(json.dumps(out))
    return 0


def cpu_baseline_leg():
    """The restatement on all host cores (2 iterations after 1 untimed) and
    on one core (1 iteration), same workload and start field."""
    from oracle import cbuild
    lib = cbuild.load()
    model, ncpu = cpu_model()
    threads = lib.scfcpu_threads()
    with cpu_context() as c:
        c.set_field(c3_fields())
        c.iterate(1)
        s_all = cpu_iterations(c, 2)
        lib.scfcpu_set_threads(1)
        try:
            s_one = cpu_iterations(c, 1)
        finally:
            lib.scfcpu_set_threads(threads)
    return {"value": 1.0 / s_all, "unit": "iter/s", "cores": threads, "kind": "port",
            "sample": f"whole SCF iterations of the same workload (2 timed after 1 untimed) on "
                      f"{threads} threads; C++17/OpenMP FP64 restatement of the reference "
                      f"(oracle/scf_cpu.cpp), {model}, nproc {ncpu}",
            "single_core_iter_s": 1.0 / s_one, "cpu_model": model, "nproc": ncpu}


# --------------------------------------------------------------------------
# batch workloads (reported beside the headline): C2 films and C5 bulk scan
# --------------------------------------------------------------------------
def c2_films(A, n=4096, seed=2, prec=None):
    """4096 symmetric diblock films: nz ~ U{64..192} tanh-clustered (2.0),
    D ~ U[2, 8], f = 0.5, chiN = 20, kappa = 25, h_A ~ U[-1, 1] as the
    amplitude of the wall potential on A, Ns ~ U{100..300} end-refined
    (half-cosine) steps, fields N(0, 0.05^2); the grand-canonical ensemble,
    mu = 2.55 and lambda mixing 0.2 of the reference's Film_1D deck; split
    precision."""
    from adscf_gb300 import mesh
    rng = np.random.default_rng(seed)
    inst, fields = [], []
    for _ in range(n):
        gz = int(rng.integers(64, 193))
        D = float(rng.uniform(2.0, 8.0))
        dz, zr = mesh.tanh_mesh(gz, D, 2.0)
        ns = int(rng.integers(100, 301))
        ns += ns % 2
        dss = mesh.contour_steps(ns, ds_scheme=1)
        h = float(rng.uniform(-1.0, 1.0))
        ext = mesh.wall_potential(zr, D, 0.4, (h, 0.0))
        inst.append(dict(geometry=A.FILM_1D, grid=(1, 1, gz), size=(1.0, 1.0, D), dz=dz, dss=dss,
                         n_a=ns // 2, block_length=(0.5, 0.5), chi=20.0, kappa=25.0,
                         ext_potential=ext, int_scheme=1, int_span=1, ensemble=2, mu=2.55,
                         precision=A.SPLIT if prec is None else prec,
                         mixing_type=A.MIX_LAMBDA, lam=0.2))
        w = rng.normal(0.0, 0.05, (2, gz + 1))
        w[:, 0] = w[:, -1] = 0.0
        fields.append(w.reshape(2, gz + 1, 1, 1))
    return inst, fields


def c5_bulk(A, n=256, seed=5, prec=None):
    """256 diblock melts: cubic grids from {24, 32, 40, 48, 64}^3, f_A ~
    U[0.25, 0.45], chiN ~ U[15, 30], L ~ U[3, 5], Ns ~ U{100..200} (ds =
    1/Ns), fields +-0.5 chiN (0.5 - f_A) cos(2 pi x / L) + N(0, 0.1^2);
    Anderson m = 10 after 10 lambda = 0.1 steps; split precision."""
    rng = np.random.default_rng(seed)
    inst, fields = [], []
    for _ in range(n):
        g = int(rng.choice([24, 32, 40, 48, 64]))
        f = float(rng.uniform(0.25, 0.45))
        chi = float(rng.uniform(15.0, 30.0))
        L_ = float(rng.uniform(3.0, 5.0))
        ns = int(rng.integers(100, 201))
        inst.append(dict(geometry=A.BULK, grid=(g, g, g), size=(L_, L_, L_), ds=1.0 / ns,
                         block_length=(round(f * ns) / ns, 1.0 - round(f * ns) / ns), chi=chi,
                         kappa=25.0, precision=A.SPLIT if prec is None else prec,
                         mixing_type=A.MIX_ANDERSON, mixing_dim=10, lam=0.1, lam_warm=0.1,
                         warm_iters=10))
        x = np.arange(g) * L_ / g
        s = np.broadcast_to(np.cos(2 * np.pi * x / L_)[None, None, :], (g, g, g))
        a = 0.5 * chi * (0.5 - f)
        fields.append(np.stack([a * s, -a * s]) + rng.normal(0.0, 0.1, (2, g, g, g)))
    return inst, fields


def oracle_fixture_parity(res, A):
    """The first iteration of both GPU paths at the C3 start field against the
    FP64 oracle's values at that field, read from the committed fixture
    tests/golden/c3_start.json (made by tests/golden/make_c3_start.py); None
    when the fixture is absent or for another configuration."""
    path = Path(__file__).resolve().parent / "tests" / "golden" / "c3_start.json"
    if not path.exists():
        return None
    fx = json.loads(path.read_text())
    if (fx["grid"], fx["L"], fx["ds"], fx["f_A"], fx["chi"], fx["kappa"], fx["seed"]) != \
            (GRID, L, DS, F_A, CHI, KAPPA, SEED):
        return None
    idx = [tuple(i) for i in fx["sample_index"]]
    ref = np.array(fx["sample_density"])
    out = {"vs": "FP64 oracle at the same field (tests/golden/c3_start.json): F per chain and log Q, "
                 "densities at 256 seeded points"}
    for prec, name in ((A.SPLIT, "split"), (A.FP64, "fp64")):
        r, d = res[prec]
        dens = np.asarray(d).reshape(2, GRID, GRID, GRID)
        out[f"dF_per_chain_{name}"] = abs(r.free_energy - fx["F"])
        out[f"dlogQ_{name}"] = abs(r.logQ - fx["logQ"])
        out[f"max_dphi_{name}"] = float(np.max(np.abs(np.array([dens[i] for i in idx]) - ref)))
    return out


def c1_parity(A):
    """C1 (the reference's CPU-runnable case: 32^3, L = 4.0, f_A = 0.30, chiN =
    kappa = 25, ds = 0.01, Anderson m = 10 after 20 lambda = 0.1 steps; start
    w = +-chiN (phi_A0 - f_A) + N(0, 0.1^2), phi_A0 = f_A + 0.1 cos(2 pi x/L),
    seed 1) converged in FP64 and in split precision on the GPU: the split
    path's own F and its FP64 evaluation at the split-converged field, each
    against the FP64 saddle."""
    n, l, f, chi = 32, 4.0, 0.30, 25.0
    rng = np.random.default_rng(1)
    x = np.arange(n) * l / n
    phi0 = f + 0.1 * np.broadcast_to(np.cos(2 * np.pi * x / l)[None, None, :], (n, n, n))
    w = np.stack([chi * (phi0 - f) + rng.normal(0.0, 0.1, (n, n, n)),
                  -chi * (phi0 - f) + rng.normal(0.0, 0.1, (n, n, n))])
    kw = dict(grid=(n, n, n), size=(l, l, l), ds=0.01, block_length=(f, 1 - f), kappa=25.0,
              chi=chi, mixing_type=A.MIX_ANDERSON, mixing_dim=10, lam=0.1, lam_warm=0.1,
              warm_iters=20)
    with A.Context(A.BULK, precision=A.FP64, **kw) as c:
        c.set_field(w)
        r64 = c.scf_run(3000, tol=1e-16)
    with A.Context(A.BULK, precision=A.SPLIT, **kw) as c:
        c.set_field(w)
        rs = c.scf_run(3000, tol=1e-8)
        pol = c.free_energy_fp64()
    return {"workload": "C1 32^3 diblock melt, converged", "fp64_iterations": r64.iter,
            "fp64_accuracy": r64.accuracy, "split_iterations": rs.iter,
            "split_accuracy": rs.accuracy,
            "dF_per_chain_split": abs(rs.free_energy - r64.free_energy),
            "dF_per_chain_split_fp64_at_split_saddle": abs(pol.free_energy - r64.free_energy),
            "vs": "FP64 GPU path converged to accuracy 1e-16"}


def c4_film3d(A, seed=4):
    """C4: AB diblock film f_A = 0.25, chiN = 30, kappa = 25, lateral 64 x 64
    periodic (L_x = L_y = 6.0), 64-interval tanh z mesh (2.0), D = 3.0, wall
    field h_A = -0.5 at the bottom wall and +0.5 at the top, Ns = 150
    end-refined contour steps; start fields a hexagonal pattern of amplitude
    0.5 plus N(0, 0.05^2); the grand-canonical ensemble, mu = 2.25 and lambda
    mixing 0.2 of the reference's Film_3D deck; Douglas ADI, split precision."""
    from adscf_gb300 import mesh
    gx = gy = 64
    gz, D, Lxy = 64, 3.0, 6.0
    dz, zr = mesh.tanh_mesh(gz, D, 2.0)
    dss = mesh.contour_steps(150, ds_scheme=1)
    lo = mesh.wall_potential(zr, D, 0.4, (1.0,), walls=(True, False))[0]
    hi = mesh.wall_potential(zr, D, 0.4, (1.0,), walls=(False, True))[0]
    ext = np.stack([-0.5 * lo + 0.5 * hi, np.zeros(gz + 1)])
    rng = np.random.default_rng(seed)
    x = np.arange(gx) * Lxy / gx
    X, Y = np.meshgrid(x, x, indexing="xy")
    k = 4 * np.pi / (np.sqrt(3.0) * Lxy / 2)
    hexp = sum(np.cos(k * (np.cos(a) * X + np.sin(a) * Y)) for a in (0.0, 2 * np.pi / 3, 4 * np.pi / 3)) / 3
    pat = np.broadcast_to(hexp[None, :, :], (gz + 1, gy, gx))
    w = np.stack([0.5 * pat, -0.5 * pat]) + rng.normal(0.0, 0.05, (2, gz + 1, gy, gx))
    w[:, 0] = w[:, -1] = 0.0
    kw = dict(grid=(gx, gy, gz), size=(Lxy, Lxy, D), dz=dz, dss=dss, n_a=int(round(0.25 * 150)),
              block_length=(0.25, 0.75), chi=30.0, kappa=25.0, ext_potential=ext,
              int_scheme=1, int_span=0, ensemble=2, mu=2.25, precision=A.SPLIT,
              mixing_type=A.MIX_LAMBDA, lam=0.2)
    return kw, w


def film3d_leg(torch, A, stream, steps):
    kw, w = c4_film3d(A)
    with A.Context(A.FILM_3D, **kw) as c:
        A._lib.check(c.lib, c.h, c.lib.adscf_set_stream(c.h, stream.cuda_stream))
        c.set_field(w)
        c._ck(c.lib.adscf_enqueue(c.h, 0, 3))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        c._ck(c.lib.adscf_enqueue(c.h, 0, steps))
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res = c.scf_run(0)
        launches = c.lib.adscf_stage_launches(c.h, 0)
        tuning = c.tuning()
    ns = len(kw["dss"]) - 1
    lines = 2 * ns * (64 * 63 + 64 * 63 + 64 * 64)   # x, y and z line solves, both chains
    return {"workload": "C4: Film_3D diblock, 64x64 lateral L=6, 64-interval tanh z mesh, D=3, "
                        "h_A -0.5/+0.5, Ns=150 end-refined, f_A=0.25, chiN=30, grand canonical mu=2.25, "
                        "ADI, split",
            "ms_per_iter": ms, "iter_s": 1000.0 / ms, "line_solves_s": lines * 1000.0 / ms,
            "contour_steps_s": 2 * ns * 1000.0 / ms, "launches_per_iter": launches,
            "accuracy": res.accuracy, "status": res.status,
            "adi_plan": tuning[tuning.index("adi"):] if "adi" in tuning else tuning}


def time_batch(torch, A, inst, fields, stream, steps, warmup):
    """Batch iterations/s over `steps` graph replays after `warmup`."""
    with A.Batch(inst) as b:
        b.set_fields(fields)
        b._ck(b.lib.adscf_batch_set_stream(b.h, stream.cuda_stream))
        b._ck(b.lib.adscf_batch_enqueue(b.h, warmup))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b._ck(b.lib.adscf_batch_enqueue(b.h, steps))
        e1.record(stream)
        torch.cuda.synchronize()
        res = (A._lib.IterResult * b.n)()
        b.lib.adscf_batch_results(b.h, res)   # status per instance, read below
        launches = b.lib.adscf_batch_launches(b.h)
    ms = e0.elapsed_time(e1) / steps
    bad = sum(1 for r in res if r.status != 0)
    return ms, launches, bad


def sharded_time(torch, A, inst, fields, stream, steps, world, rank):
    """Time this rank's share of a batch (contiguous, cost-balanced instance
    range, no collective on the data path); the batch time is the maximum
    over ranks."""
    from adscf_gb300 import parallel
    if world == 1:
        return time_batch(torch, A, inst, fields, stream, steps, 3)
    rg = parallel.shard([parallel.instance_cost(k) for k in inst], rank, world)
    ms, launches, bad = 0.0, 0, 0
    if len(rg):
        ms, launches, bad = time_batch(torch, A, [inst[i] for i in rg], [fields[i] for i in rg],
                                       stream, steps, 3)
    ms = parallel.max_over_ranks(ms, device="cuda")
    return ms, launches, bad


def batch_legs(torch, A, stream, args, world=1, rank=0):
    """C2 and C5 batches; with several ranks each rank runs its instance
    range and the figures are whole-batch throughputs."""
    out = {}
    inst, fields = c2_films(A)
    ms, launches, bad = sharded_time(torch, A, inst, fields, stream, args.batch_steps, world, rank)
    pts_steps = sum(2 * len(k["dss"]) * (k["grid"][2] + 1) for k in inst)   # both chains
    out["film_batch"] = {
        "workload": "C2: 4096 Film_1D diblock films, nz 64-192 tanh meshes, D 2-8, Ns 100-300 "
                    "end-refined, h_A in [-1,1], grand canonical mu=2.55, split precision, "
                    "lambda mixing 0.2",
        "films": len(inst), "ms_per_iter": ms, "iter_s": 1000.0 / ms,
        "film_iter_s": len(inst) * 1000.0 / ms,
        "line_solves_s": 2 * len(inst) * sum(len(k["dss"]) - 1 for k in inst) / len(inst) * 1000.0 / ms,
        "point_steps_s": pts_steps * 1000.0 / ms,
        "launches_per_iter": launches, "nonfinite_instances": bad,
        "sharding": f"{world} rank(s), contiguous cost-balanced instance ranges"}
    inst, fields = c5_bulk(A)
    ms, launches, bad = sharded_time(torch, A, inst, fields, stream, args.batch_steps, world, rank)
    steps = sum(2 * round(1.0 / k["ds"]) for k in inst)
    out["bulk_batch"] = {
        "workload": "C5: 256 bulk diblock instances, grids {24,32,40,48,64}^3, f_A 0.25-0.45, "
                    "chiN 15-30, L 3-5, Ns 100-200, split precision, Anderson m=10",
        "instances": len(inst), "ms_per_iter": ms, "iter_s": 1000.0 / ms,
        "instance_iter_s": len(inst) * 1000.0 / ms, "contour_steps_s": steps * 1000.0 / ms,
        "launches_per_iter": launches, "nonfinite_instances": bad,
        "sharding": f"{world} rank(s), contiguous cost-balanced instance ranges"}
    return out


def run_profile_workload(name, adi_plan=None):
    """One SCF iteration of a film or batch workload for a launch list:
    c4 (Film_3D, 64 x 64 x 65, ADI), c2 (4096 films), c5 (256 bulk
    instances), after two untimed iterations.  For c4 the ADI plan in use is
    printed as "adi plan x,y,z,mask" (mask: 2 y staged, 4 z staged, 8 x and
    y fused); ``adi_plan`` pins one (with
    ADSCF_AUTOTUNE=0 the context skips the tuner's candidate launches, whose
    timings mean nothing under a profiler)."""
    import adscf_gb300 as A
    if name == "c4":
        kw, w = c4_film3d(A)
        with A.Context(A.FILM_3D, **kw) as c:
            if adi_plan:
                c.set_adi_plan(*adi_plan)
            rep = c.tuning()
            c.set_field(w)
            c.scf_run(3)
        import re
        chosen = dict((a, (int(g), st)) for a, g, _, st in
                      re.findall(r"\b([xyz])=(\d+)x(\d+)(s?)", rep[rep.index("adi"):])) if "adi" in rep else {}
        if adi_plan:
            print("adi plan " + ",".join(str(v) for v in adi_plan))
        elif chosen:
            mask = (2 if chosen["y"][1] else 0) + (4 if chosen["z"][1] else 0) + (8 if "xy=fused" in rep else 0)
            print(f"adi plan {chosen['x'][0]},{chosen['y'][0]},{chosen['z'][0]},{mask}")
    else:
        inst, fields = c2_films(A) if name == "c2" else c5_bulk(A)
        with A.Batch(inst) as b:
            b.set_fields(fields)
            b.scf_run(3)
    print(f"profile run {name} done")
    return 0


def run_profile(pass_plan=None):
    """One SCF iteration's stages at 128^3, ds = 0.05 (20 contour steps, 340 MB
    of slices) on the split path: the kernels of the bench, few launches.
    ``pass_plan`` (y, z, x) pins the pass kernels (with ADSCF_AUTOTUNE=0 the
    context skips the tuner's candidate launches)."""
    import adscf_gb300 as A
    from adscf_gb300 import _lib as L_
    w = c3_fields()
    c = A.Context(A.BULK, grid=(GRID, GRID, GRID), size=(L, L, L), ds=0.05,
                  block_length=(F_A, 1.0 - F_A), kappa=KAPPA, chi=CHI, precision=A.SPLIT,
                  mixing_type=A.MIX_ANDERSON, mixing_dim=M_HIST, lam=LAM, lam_warm=LAM,
                  warm_iters=M_HIST)
    if pass_plan:
        c.set_pass_plan(*pass_plan)
    c.set_field(w)
    for st in (L_.STAGE_PROPAGATE, L_.STAGE_CONTOUR, L_.STAGE_UPDATE):
        c._ck(c.lib.adscf_enqueue(c.h, st, 1))
    c.get_field()
    c.close()
    print("profile run done")
    return 0


# --------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-batches", action="store_true", help="skip the C2 / C5 batch legs")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--saddle-iters", type=int, default=800,
                    help="split-path iterations toward the saddle for the converged parity")
    ap.add_argument("--profile", nargs="?", const="bulk", default=None,
                    choices=["bulk", "c4", "c2", "c5"],
                    help="small run for ncu: bulk (default) = one propagation, contour and "
                         "update of the split path at 128^3 with 20 contour steps; c4 / c2 / c5 = "
                         "three SCF iterations of that workload")
    ap.add_argument("--pass-plan", default=None,
                    help="with --profile: pin the Y, Z, X pass kernels, e.g. 2,2,3 "
                         "(0 plain, 1 persistent, 2 TMA, 3 fused XY)")
    ap.add_argument("--adi-plan", default=None,
                    help="with --profile c4: pin the ADI sweeps' lanes per line x,y,z and the "
                         "staging mask (2 y, 4 z), e.g. 16,16,16,6")
    args = ap.parse_args()
    if args.profile:
        if args.profile != "bulk":
            adi = tuple(int(v) for v in args.adi_plan.split(",")) if args.adi_plan else None
            return run_profile_workload(args.profile, adi)
        plan = tuple(int(v) for v in args.pass_plan.split(",")) if args.pass_plan else None
        return run_profile(plan)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import adscf_gb300 as A
    from adscf_gb300 import _lib as L_

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    w = c3_fields()
    nv = w.size
    npts = GRID ** 3

    # ---- parity at the same field: split vs FP64 (untimed) -------------
    res = {}
    for prec in (A.FP64, A.SPLIT):
        with make_ctx(A, prec, stream) as c:
            c.set_field(w)
            x1, d1, r1 = c.scf_iteration(w.reshape(-1))
            res[prec] = (r1, d1)
    dF = abs(res[A.SPLIT][0].free_energy - res[A.FP64][0].free_energy)
    dphi = float(np.max(np.abs(res[A.SPLIT][1] - res[A.FP64][1])))
    dlogQ = abs(res[A.SPLIT][0].logQ - res[A.FP64][0].logQ)
    par_oracle = oracle_fixture_parity(res, A)

    # ---- FP64 GPU path timing ---------------------------------------------
    with make_ctx(A, A.FP64, stream) as c64:
        c64.set_field(w)
        c64.scf_run(M_HIST + 1)                     # past the warm-up mixing
        time_stage(torch, c64, stream, L_.STAGE_ITERATION, 1)
        t64 = time_stage(torch, c64, stream, L_.STAGE_ITERATION, args.fp64_steps)
    fp64_iter_s = 1000.0 / t64

    # ---- split path: the timed region ------------------------------------
    ctx = make_ctx(A, A.SPLIT, stream)
    ctx.set_field(w)
    ctx.scf_run(M_HIST + 1)                         # Anderson active from here
    lib = ctx.lib
    ctx._ck(lib.adscf_enqueue(ctx.h, L_.STAGE_ITERATION, args.warmup))
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    ctx._ck(lib.adscf_enqueue(ctx.h, L_.STAGE_ITERATION, args.steps))
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    if dist:
        from adscf_gb300.parallel import max_over_ranks
        ms_total = max_over_ranks(ms_total, device="cuda")
    ms_step = ms_total / args.steps
    launches_per_step = lib.adscf_stage_launches(ctx.h, L_.STAGE_ITERATION)
    pass_plan = ctx.tuning()

    # ---- stage breakdown (CUDA events on the launching stream) ------------
    ns = ctx.ns
    t_prop = time_stage(torch, ctx, stream, L_.STAGE_PROPAGATE, 3)
    t_cont = time_stage(torch, ctx, stream, L_.STAGE_CONTOUR, 3)
    t_upd = time_stage(torch, ctx, stream, L_.STAGE_UPDATE, 3)
    t_dstep = t_prop / ns                            # one double step (q and q-dagger)
    alg_dstep = 2 * 12 * npts                        # 12 N B per propagator step, two chains
    hbm, peak_kind = peaks()
    achieved = alg_dstep / (t_dstep * 1e-3) / 1e9
    alg_contour = 8 * (ns + 1) * npts + 16 * npts   # read all FP32 slices, write FP64 phi
    l2_peak = L_.c_double_out(lib.adscf_probe_l2_copy, 24 << 20, 50)

    # ---- end to end through the C ABI with host buffers ---------------------
    # page-locked host buffers: the call copies them by DMA directly
    xh = torch.empty(nv, dtype=torch.float64, pin_memory=True).numpy()
    xh[:] = w.reshape(-1)
    dh = torch.empty(nv, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):
        xh, dh, _r = ctx.scf_iteration(xh, dh, inplace=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ke2e = max(3, args.steps // 2)
    for _ in range(ke2e):
        xh, dh, _r = ctx.scf_iteration(xh, dh, inplace=True)
    e2e_s = (time.perf_counter() - t0) / ke2e

    # ---- parity at a converged field (untimed) ------------------------------
    # F is stationary in the densities at a saddle point, so the FP32 density
    # error drops out to first order there; converge the split path, then
    # evaluate both precisions at the same field
    ctx.set_field(xh)
    conv = ctx.scf_run(args.saddle_iters if world == 1 else 0, tol=1e-12)
    ws = ctx.get_field()
    _x, ds_, rs = ctx.scf_iteration(ws.copy())
    with make_ctx(A, A.FP64, stream) as c64:
        _x, dd_, rd = c64.scf_iteration(ws.copy())
    saddle = {"dF_per_chain": abs(rs.free_energy - rd.free_energy),
              "dlogQ": abs(rs.logQ - rd.logQ),
              "max_dphi": float(np.max(np.abs(ds_ - dd_))),
              "accuracy": conv.accuracy, "iterations": conv.iter,
              "vs": "FP64 GPU path, same converged field"}
    ctx.close()

    value = world * 1000.0 / ms_step
    out = {
        "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32/f64-split", "data": "synthetic",
        "config": config(world),
        "fp64_gpu_iter_s": world * fp64_iter_s,
        "split_over_fp64": fp64_iter_s and (1000.0 / ms_step) / fp64_iter_s,
        "contour_steps_per_s": world * 2 * ns * 1000.0 / ms_step,
        "parity": {"dF_per_chain": dF, "max_dphi": dphi, "dlogQ": dlogQ,
                   "vs": "FP64 GPU path, same field (the bench's start iterate), one iteration"},
        "parity_oracle": par_oracle,
        "parity_saddle": saddle,
        "stages_ms": {"propagate": t_prop, "contour": t_cont, "update": t_upd,
                      "double_step": t_dstep},
        "roofline": {"bound": "hbm", "kernel": "propagator double step (Yf, Z, Yi, X passes)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind,
                     "algorithmic_bytes": alg_dstep, "traffic": DSTEP_TRAFFIC,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum summed "
                                       "over the four passes of one 128^3 double step "
                                       "(--cache-control none; Boltzmann factors and spectrum "
                                       "stay in L2, only the slice store reaches DRAM)",
                     "contour_GBs": alg_contour / (t_cont * 1e-3) / 1e9,
                     "l2": {"bytes_per_double_step": DSTEP_L2_BYTES,
                            "achieved_gbs": DSTEP_L2_BYTES / (t_dstep * 1e-3) / 1e9,
                            "peak_gbs": l2_peak,
                            "frac": (DSTEP_L2_BYTES / (t_dstep * 1e-3) / 1e9) / l2_peak if l2_peak else None,
                            "peak_source": "adscf_probe_l2_copy: copy of two 24 MiB buffers "
                                           "(L2-resident), read + write bytes",
                            "bytes_source": "ncu lts__t_sectors_srcunit_tex.sum x 32 B, one launch "
                                            "each of the XY and Z passes at 128^3"}},
        "pass_plan": pass_plan,
        "clocks": clk,
        "gpu_launches": launches_per_step * args.steps,
        "e2e": {"value": world / e2e_s, "unit": "iter/s", "h2d_bytes_per_step": nv * 8,
                "d2h_bytes_per_step": 2 * nv * 8 + 13 * 8,
                "api": "adscf_scf_iteration (page-locked host field in/out, host density out)"},
    }
    if world == 1:
        out["parity_c1"] = c1_parity(A)
    if not args.no_batches:
        if world == 1:
            out["film3d"] = film3d_leg(torch, A, stream, args.batch_steps)
        out.update(batch_legs(torch, A, stream, args, world, rank))
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_leg()
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
