#!/usr/bin/env python
"""Throughput benchmark: atom-force evaluations per second on one GB300.

Workload (one "step"): a batch of B seeded ternary-alloy structures of 512
atoms each (fcc 4x4x8, a = 3.9 A, Z = 13/28/40 at 0.5/0.3/0.2, jitter
0.08 A), wACSF D = 64 (20 radial + 12 angular SFs, zeta 1/2/4), sparse GPR
with M = 4000 points (theta = 0.8 std, coeff ~ N(0, 1e-3)); every step
produces energy, forces and stress of all B*512 atoms.  Synthetic data, no
dataset.  "value" is measured with inputs resident in HBM (device-buffer
C-ABI call on the launching stream, CUDA events, L2 flushed between steps);
"e2e" through the host-buffer C-ABI call with pinned host inputs, host<->device
copies inside the timed region.  The precision form measured is the chosen
fast form; the plain FP64 path is timed beside it, and both are compared
with the FP64 oracle on one structure.

--impl reference times the CPU restatement of the reference (the oracle,
single-threaded per structure as the reference is) on all host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "calypso-gap_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "atom-force evals/s on 1 GB300: chosen vs plain GPU at <=1 meV/atom, <=20 meV/A"
UNIT = "atoms/s"
ATOMS = 512
M_SPARSE = 4000
L2_FLUSH_BYTES = 512 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gapgb", choices=["gapgb", "reference"])
    p.add_argument("--batch", type=int, default=None,
                   help="structures per step per GPU (default: one full wave of the tensor-core "
                        "GPR, two 128-atom CTAs per SM: 76 alloy512 cells on 152 SMs)")
    p.add_argument("--precision", default="tc", choices=["fp32", "tc", "tf32", "fp64", "mixed"])
    p.add_argument("--no-oracle", action="store_true", help="skip the oracle error check")
    p.add_argument("--pipelines", type=int, default=2, choices=[1, 2],
                   help="alloy workload: GAPGB_OPT_PIPELINES of the timed model (2: a large "
                        "tensor-core batch runs as two halves on two streams)")
    p.add_argument("--workload", default="alloy", choices=["alloy", "population", "surrogate", "md", "precision",
                                             "variance", "fit"],
                   help="alloy: 512-atom ternary fcc cells (the headline metric); population: "
                        "a ragged structure-search population evaluated by one CUDA graph; "
                        "surrogate: the learned surrogate with GPR fallback on held-out alloy "
                        "cells, after training on GAP labels; md: 32768-atom Si/Ge NVE "
                        "velocity Verlet, tensor-core form against the plain FP64 path; "
                        "precision: the alloy step in every arithmetic form (FP64, FP32, "
                        "mixed, TF32, split-BF16x3) with each form's error; variance: the "
                        "GPR variance block (qmm attached) on the alloy workload; fit: the "
                        "coefficients refitted from teacher energies of --fit-structs cells")
    p.add_argument("--count", type=int, default=8192,
                   help="population size / held-out structures of the surrogate workload")
    p.add_argument("--train-structs", type=int, default=20000,
                   help="surrogate workload: training structures (512 atoms each)")
    p.add_argument("--epochs", type=int, default=4, help="surrogate workload: training epochs")
    p.add_argument("--fit-structs", type=int, default=512,
                   help="fit workload: training cells (512 atoms each)")
    p.add_argument("--md-steps", type=int, default=100, help="md workload: velocity-Verlet steps")
    p.add_argument("--md-reps", type=int, default=16,
                   help="md workload: diamond cells per axis (16: 32768 atoms; smaller for profiling)")
    p.add_argument("--threshold", type=float, default=0.005,
                   help="surrogate workload: committee std (eV) above which an atom takes the GPR")
    p.add_argument("--contact", type=float, default=None,
                   help="surrogate workload: neighbour distance (A) below which an atom takes "
                        "the GPR (default: the 0.2%% quantile of the training cells' nearest-"
                        "neighbour distances; 0 = off)")
    p.add_argument("--surrogate-theta", type=float, default=4.0,
                   help="surrogate workload: theta of the GAP in units of std(MM) (4: the smooth "
                        "alloy GAP; 0.8: the throughput workload's GAP)")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def shard_seeds(rank, batch):
    """Seeds of rank `rank`'s structures: disjoint blocks of `batch` seeds, so
    N ranks evaluate N x batch different cells (weak scaling, no data-path
    collective)."""
    return [100000 + rank * batch + s for s in range(batch)]


def default_batch(args, device):
    """Structures per step: by default one full wave of the tensor-core GPR
    kernel, which holds 128 atoms per CTA and two CTAs per SM (76 alloy512
    cells = 38912 atoms on 152 SMs)."""
    if args.batch is None:
        import torch
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        args.batch = max(1, sms * 2 * 128 // ATOMS)
    return args.batch


def workload(rank, batch):
    import gapgb.synth as S
    structs = [S.alloy512(seed=sd) for sd in shard_seeds(rank, batch)]
    return structs, S.pack(structs)


def max_over_ranks(x, world, device):
    """The largest value of x over all ranks (the job's time is its slowest
    rank's); the only collective of the benchmark."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def make_model():
    """The synthetic alloy model: sparse points are descriptors of 8 seeded
    alloy cells computed by the library itself."""
    import gapgb
    import gapgb.synth as S
    ty, al, rc, ze = S.sf_table()
    zt = np.array([13, 28, 40], np.int32)
    wt = zt.astype(np.float64)
    D = 2 * len(ty)
    probe = gapgb.GapModel.create(zt, wt, ty, al, rc, np.ones(D), np.zeros((1, D)), np.zeros(1),
                                  sf_zeta=ze)
    cells = [S.alloy512(seed=s) for s in range(8)]
    off, sp, lat, pos = S.pack(cells)
    X = probe.descriptors(off, sp, lat, pos)
    probe.close()
    theta, mm, coeff = S.model_arrays(X, M_SPARSE, theta_scale=0.8, coeff_std=1e-3, seed=0)
    arrays = (zt, wt, ty, al, rc, ze, theta, mm, coeff)
    return arrays


def clocks_sampler(stop, out):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    dev = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0] or "0"
    try:
        p = subprocess.Popen(["nvidia-smi", "-i", dev, "--query-gpu=" + q,
                              "--format=csv,noheader,nounits", "-lms", "100"],
                             stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except (FileNotFoundError, OSError):
        return
    stop.wait()
    p.terminate()
    try:
        txt, _ = p.communicate(timeout=5)
    except subprocess.TimeoutExpired:
        p.kill()
        txt = ""
    out.extend(l for l in txt.splitlines() if l.strip())


def summarize_clocks(lines):
    if not lines:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    sm, smax, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for l in lines:
        f = [x.strip() for x in l.split(",")]
        try:
            sm.append(float(f[1]))
            smax = float(f[2])
        except (ValueError, IndexError):
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
            "reasons": sorted(reasons), "samples": len(sm)}


def oracle_errors(arrays, structs, results):
    """Max |dE|/atom (eV) and max |dF| (eV/A) of GPU results vs the FP64 oracle
    on the first structure of the batch."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import write_model_file
    from oracle import oracle
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    with tempfile.TemporaryDirectory() as d:
        path = write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta, mm, coeff, ze)
        om = oracle.Model(path)
        lat, pos, z = structs[0]
        oE, oF, oS, _ = oracle.gap_calc(om, z, lat, pos, 6.0, True)
    out = {}
    for name, (E, F, St) in results.items():
        out[name] = {"dE_per_atom_eV": abs(E[0] - oE) / len(pos),
                     "max_dF_eV_per_A": float(np.abs(F[:len(pos)] - oF).max()),
                     "max_dstress_GPa": float(np.abs(St[0] - oS).max())}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import tempfile
    from helpers import write_model_file
    # the same model arrays the GPU arm builds (descriptors from the oracle here)
    import gapgb.synth as S
    ty, al, rc, ze = S.sf_table()
    zt = np.array([13, 28, 40], np.int32)
    wt = zt.astype(np.float64)
    D = 2 * len(ty)
    cores = len(os.sched_getaffinity(0))
    with tempfile.TemporaryDirectory() as d:
        probe = write_model_file(os.path.join(d, "probe"), zt, wt, ty, al, rc, np.ones(D),
                                 np.zeros((1, D)), np.zeros(1), ze)
        pm = oracle.Model(probe)
        X = []
        for s in range(8):
            lat, pos, z = S.alloy512(seed=s)
            cnt, nb = oracle.neighbors(lat, pos, pm.weights(z), 6.0, 400)
            X.append(oracle.car2acsf(pm, pos, cnt, nb)[0])
        theta, mm, coeff = S.model_arrays(np.concatenate(X), M_SPARSE, 0.8, 1e-3, 0)
        path = write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta, mm, coeff, ze)
        om = oracle.Model(path)
        structs = [S.alloy512(seed=100000 + s) for s in range(cores)]
        off, sp, lat, pos = S.pack(structs)
        times = []
        for it in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            oracle.gap_calc_batch(om, off, sp, lat, pos, 6.0, cores)
            dt = time.perf_counter() - t0
            if it >= args.warmup:
                times.append(dt)
    atoms = cores * ATOMS
    v = atoms * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "alloy512 ternary fcc, D=64, M=4000", "atoms_per_structure": ATOMS,
                   "structures_per_step": cores, "model": "synthetic sparse GPR"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d alloy512 structures per step, one per host thread "
                                   "(CPU FP64 restatement, dense Jacobian as the reference)" % cores},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(arrays):
    """The oracle on the host cores on a bounded sample (one alloy512
    structure per core), plus the latency of one structure on one core (the
    reference is single-threaded and farmed one structure per process)."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import write_model_file
    from oracle import oracle
    import gapgb.synth as S
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    cores = len(os.sched_getaffinity(0))
    with tempfile.TemporaryDirectory() as d:
        om = oracle.Model(write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta, mm,
                                           coeff, ze))
        structs = [S.alloy512(seed=100000 + s) for s in range(cores)]
        off, sp, lat, pos = S.pack(structs)
        t0 = time.perf_counter()
        oracle.gap_calc_batch(om, off, sp, lat, pos, 6.0, cores)
        dt = time.perf_counter() - t0
        off1, sp1, lat1, pos1 = S.pack(structs[:1])
        t0 = time.perf_counter()
        oracle.gap_calc_batch(om, off1, sp1, lat1, pos1, 6.0, 1)
        lat_s = time.perf_counter() - t0
    return {"value": cores * ATOMS / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d alloy512 structures (one per host thread), %.1f s" % (cores, dt),
            "latency_1core_s": lat_s,
            "latency_sample": "one alloy512 structure (E, F, stress) on one host thread"}


def dropin_latency(reps=30):
    """Latency of one evaluation as the reference is used: one structure per
    ASE call (gappy/ASE/gap_calc.py:29-52, gappy/example/ASE-GAPPY/run_md.py:
    10-21).  The reference's own example model and the first frame of its MD
    trajectory (64-atom C diamond, committed under tests/golden), plain FP64
    path, median milliseconds per call after two warm-up calls:
      ase_calculate    ase_gap.GAP.calculate (a new libgap Calculator per
                       call, as the reference builds one; the file is read
                       and the device model reused while it is unchanged)
      libgap_gap_calc  libgap.GAP.Calculator.gap_calc
      c_abi_eval       gapgb_eval with host buffers
    and beside them the oracle (the CPU restatement of FGAP_CALC) on one host
    core on the same frame.  first_call_ms is the first ASE call of the
    process (model upload, workspace allocation)."""
    import shutil
    import tempfile
    import gapgb
    from oracle import oracle
    golden = os.path.join(ROOT, "tests", "golden")
    fr = np.load(os.path.join(golden, "ase_traj_frames.npz"))
    z, lat, pos = fr["numbers"][0], fr["cell"][0], fr["positions"][0]

    class Atoms:  # the part of ase.Atoms the calculator reads
        def __init__(self, z, cell, pos):
            self.numbers, self.cell, self.positions = z, cell, pos

        def get_atomic_numbers(self):
            return self.numbers

        def copy(self):
            return Atoms(self.numbers.copy(), self.cell.copy(), self.positions.copy())

    def median_ms(fn, n):
        ts = []
        for _ in range(n):
            t0 = time.perf_counter()
            fn()
            ts.append((time.perf_counter() - t0) * 1e3)
        return float(np.median(ts))

    cwd = os.getcwd()
    d = tempfile.mkdtemp()
    try:
        shutil.copy(os.path.join(golden, "gap_parameters_c_diamond"),
                    os.path.join(d, "gap_parameters"))
        os.chdir(d)
        from ase_gap.gap_calc import GAP
        from libgap.GAP import Calculator
        atoms = Atoms(z, lat, pos)
        calc = GAP(rcut=6.0)
        t0 = time.perf_counter()
        calc.calculate(atoms, ["energy", "forces", "stress"])
        first = (time.perf_counter() - t0) * 1e3
        out = {"first_call_ms": first}
        for _ in range(2):
            calc.calculate(atoms, ["energy", "forces", "stress"])
        out["ase_calculate"] = median_ms(
            lambda: calc.calculate(atoms, ["energy", "forces", "stress"]), reps)
        c = Calculator(rcut=6.0)
        c.gap_calc(z, lat, pos, True)
        out["libgap_gap_calc"] = median_ms(lambda: c.gap_calc(z, lat, pos, True), reps)
        m = gapgb.GapModel.load("gap_parameters")
        m.eval(z, lat, pos)
        m.eval(z, lat, pos)
        out["c_abi_eval"] = median_ms(lambda: m.eval(z, lat, pos), reps)
        m.close()
        oracle.build()
        om = oracle.Model("gap_parameters")
        out["oracle_1core"] = median_ms(lambda: oracle.gap_calc(om, z, lat, pos, 6.0, True), 3)
    finally:
        os.chdir(cwd)
        shutil.rmtree(d, ignore_errors=True)
    out["sample"] = ("reference example model (M = 129, D = 66), ase.traj frame 0: 64 C "
                     "atoms, 158 neighbours per atom; E, F and stress per call")
    return out


STAGES = ["neighbours", "descriptors", "gpr", "chain_rule"]
# algorithmic HBM bytes per atom of each stage's kernels (P = 56 neighbour
# slots per atom on this workload, D = 64, FP32 slot records):
#   neighbours : positions in, slot records out per slot (j 4, shift 4,
#                FP32 record 16, weight 4)
#   descriptors: FP32 slot record + weight in per slot, D FP32 descriptors
#                out, and the contributing angular pairs out (2 B each)
#   chain_rule : slot record + weight + partner index in per slot, the pair
#                list in, dE/dG row in, per-atom virial (72 B) out, and the
#                force scatter: 24 B (an FP64 atomic add per component) per
#                slot and per atom
P_SLOTS = 56.0
T_PAIRS = 690.0  # contributing angular pairs per atom on this workload


def step_kernels(precision, natoms, generic=False, pipelines=2):
    """Kernels the library launches per evaluation with gradients: prep x2
    and the two neighbour-build kernels (cells wider than twice the cutoff,
    then the others; the one with no cell of its kind returns at once); per
    pipeline the descriptors, the GPR (tensor-core
    forms: operand prep + kernel; SIMT forms: kernel + split reduce) and the
    slot gradients (the grouped kernel scatters the forces itself); then the
    structure partial and final sums.  Tensor-core batches of at least the
    library's split threshold run two pipelines; the generic descriptor
    kernels add the reverse slots, the force gather and the orphans."""
    from gapgb.tune import SPLIT_MIN_ATOMS
    two = (pipelines == 2 and precision in ("tc", "tf32") and not generic
           and natoms >= SPLIT_MIN_ATOMS)
    return 4 + 4 * (2 if two else 1) + 2 + (3 if generic else 0)


def stage_bytes_per_atom(D, P=P_SLOTS, T=T_PAIRS):
    return {"neighbours": 32.0 + P * 28.0,
            "descriptors": P * 20.0 + D * 4.0 + T * 2.0,
            "gpr": D * 4.0 * 2 + 8.0,
            "chain_rule": P * 24.0 + T * 2.0 + D * 4.0 + 72.0 + P * 24.0 + 24.0}


def load_peaks():
    """The measured denominators (MEASURED_PEAKS.json) or the fallback."""
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        return json.load(open(peaks_path)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def measure_tf32_tflops(n=8192, reps=10):
    """Dense TF32 rate of this device: a cuBLAS FP32 GEMM with TF32 tensor-core
    math (torch.matmul, n x n x n), CUDA events after warm-up."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        g = torch.Generator(device="cuda").manual_seed(0)
        a = torch.randn(n, n, device="cuda", generator=g)
        b = torch.randn(n, n, device="cuda", generator=g)
        for _ in range(3):
            torch.matmul(a, b)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        return 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def roofline(stages, N, D, precision, simt=None, plain_stages=None, P=P_SLOTS, T=T_PAIRS,
             traffic_file=True, tf32_tflops=None):
    """Roofline entries from the per-stage device times (ms per step).

    `simt` holds the measured FP32 / FP64 FMA and MUFU ex2 rates of the device
    (gapgb.measure_peaks); `plain_stages` the stage times of the plain FP64
    path on the same workload; P and T the workload's slots and contributing
    angular pairs per atom; `traffic_file` reads the DRAM bytes per atom of
    the alloy512 capture (only meaningful on that workload)."""
    peaks, src = load_peaks()
    dom = int(np.argmax(stages))
    name = STAGES[dom]
    bpa = stage_bytes_per_atom(D, P, T)
    ach = bpa[name] * N / (stages[dom] * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "roofline_inputs.txt")
    if traffic_file and os.path.exists(tpath):
        per_atom = json.load(open(tpath)).get("dram_bytes_per_atom", {}).get(name)
        if per_atom is not None:
            traffic = per_atom * N
    roof = {"kernel": name, "bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": ach / peaks["hbm_gbs"], "traffic": traffic,
            "peak_source": src + " hbm_gbs",
            "note": "descriptor-side kernels are FP32-pipe bound; descriptors_fp32 and "
                    "chain_rule_fp32 give their arithmetic rate against the measured FP32 "
                    "FMA rate",
            "stage_ms": {n: float(s) for n, s in zip(STAGES, stages)},
            "stage_ms_note": "library stage events on one stream (the profiling path runs the "
                             "stages in sequence); a timed tensor-core step of 20480 atoms or "
                             "more runs two pipelines, so it is shorter than their sum",
            "algorithmic_bytes_per_atom": bpa[name]}
    # FP32 arithmetic of the chain-rule / descriptor kernels (counted FLOPs per
    # angular pair and radial term, 32 SFs) against the measured FP32 FMA rate
    # (fallback: 152 SMs x 128 lanes x 2 x 2.07 GHz)
    nominal_fp32 = 152 * 128 * 2 * 2.07e9 / 1e12
    fp32_peak = simt["fp32_tflops"] if simt else nominal_fp32
    fp32_src = "measured fp32 FMA (gapgb_measure_peaks)" if simt else "nominal"
    if simt:
        roof["simt_peaks"] = simt
    m = M_SPARSE
    if precision == "tc":
        mp = ((m + 127) // 128) * 128
        npad = ((N + 127) // 128) * 128
        hw = 12.0 * npad * mp * 64  # 2 GEMMs x 3 split products x 2 flops (padded)
        ach_t = hw / (stages[2] * 1e-3) / 1e12
        roof["gpr_tensor"] = {"bound": "tensor", "achieved": ach_t, "peak": peaks["bf16_tflops"],
                              "unit": "TFLOP/s", "frac": ach_t / peaks["bf16_tflops"],
                              "peak_source": src + " bf16_tflops",
                              "flops": "12 N M 64 (bf16 MMA, padded to 128)"}
    elif precision == "tf32":
        mp = ((m + 63) // 64) * 64
        npad = ((N + 127) // 128) * 128
        hw = 4.0 * npad * mp * 64  # 2 GEMMs x 1 product x 2 flops (padded)
        ach_t = hw / (stages[2] * 1e-3) / 1e12
        if tf32_tflops:
            pk, psrc = tf32_tflops, "measured cuBLAS TF32 GEMM (torch.matmul 8192^3) on this device"
        else:
            pk = 0.5 * peaks["bf16_tflops"]
            psrc = src + " bf16_tflops x 0.5 (the nominal TF32:BF16 dense ratio)"
        roof["gpr_tensor"] = {"bound": "tensor", "achieved": ach_t, "peak": pk,
                              "unit": "TFLOP/s", "frac": ach_t / pk, "peak_source": psrc,
                              "flops": "4 N M 64 (tf32 MMA, padded)"}
    roof["gpr_algorithmic_tflops"] = 4.0 * m * D * N / (stages[2] * 1e-3) / 1e12
    roof["fp32_nominal_tflops"] = nominal_fp32
    # the GPR's exp rate (one per atom and sparse point) against the measured
    # MUFU ex2 rate (fallback: 16 per SM per clock)
    exps = N * m / (stages[2] * 1e-3)
    mufu = simt["ex2_per_s_1e12"] * 1e12 if simt else 152 * 16 * 2.07e9
    roof["gpr_exp"] = {"per_s": exps, "peak_per_s": mufu, "frac": exps / mufu,
                       "peak_source": "measured ex2.approx" if simt else "nominal"}
    # FP32 arithmetic of the descriptor-side stages, counted per contributing
    # angular pair and per (slot, radial SF) with the grouped formulation's
    # flops (an FMA = 2): forward 70 per pair (geometry 10, the NAL exponential
    # factors 6, fc(r_jk) 4, Bernstein basis 10, 2 x NAL x 5 moment FMAs 40)
    # and 8 per radial term; gradient 150 per pair and 15 per radial term
    R = 20
    fl_fwd = N * (70.0 * T + 8.0 * P * R)
    fl_bwd = N * (150.0 * T + 15.0 * P * R)
    for name, fl, st in (("descriptors_fp32", fl_fwd, stages[1]), ("chain_rule_fp32", fl_bwd, stages[3])):
        ach = fl / (st * 1e-3) / 1e12
        roof[name] = {"achieved_tflops": ach, "peak_tflops": fp32_peak,
                      "peak_source": fp32_src, "frac": ach / fp32_peak,
                      "flops_per_atom": fl / N}
    if plain_stages is not None:
        # the plain FP64 path: GPR 4 M D flops per atom (two N x M x D
        # contractions) and the descriptor / chain-rule stages with the same
        # counted flops as above, all against the measured FP64 FMA rate
        fp64_peak = simt["fp64_tflops"] if simt else None
        pl = {"stage_ms": {n: float(x) for n, x in zip(STAGES, plain_stages)},
              "peak_tflops": fp64_peak,
              "peak_source": "measured fp64 FMA (gapgb_measure_peaks)" if simt else None}
        for name, fl, st in (("gpr", 4.0 * m * D * N, plain_stages[2]),
                             ("descriptors", fl_fwd, plain_stages[1]),
                             ("chain_rule", fl_bwd, plain_stages[3])):
            ach = fl / (st * 1e-3) / 1e12
            pl[name] = {"achieved_tflops": ach,
                        "frac": ach / fp64_peak if fp64_peak else None}
        roof["plain_fp64"] = pl
    return roof


def _population_chunk(args):
    seed, count = args
    import gapgb.synth as S
    return S.population(count, seed=seed)


def build_population(count, seed=7, workers=None):
    """Seeded population (8-256 atoms, 1-4 species from {3, 8, 14, 26},
    12-20 A^3/atom, triclinic 60-120 deg, min distance 1.6 A), generated in
    parallel by a spawn-started process pool (no CUDA state is inherited)."""
    import multiprocessing as mp
    import gapgb.synth as S
    workers = workers or max(1, min(16, len(os.sched_getaffinity(0))))
    chunk = (count + workers - 1) // workers
    jobs = [(seed * 1000 + w, min(chunk, count - w * chunk)) for w in range(workers)
            if count - w * chunk > 0]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_population_chunk, jobs)
    offs, sps, lats, poss = [], [], [], []
    base = 0
    for off, sp, lat, pos in parts:
        offs.append(off[:-1] + base)
        base += int(off[-1])
        sps.append(sp), lats.append(lat), poss.append(pos)
    off = np.concatenate(offs + [np.array([base])]).astype(np.int32)
    return off, np.concatenate(sps), np.concatenate(lats), np.concatenate(poss)


def run_population(args):
    """One CUDA-graph launch evaluates the whole ragged population; the
    configuration (precision form, kernel family, neighbour capacity) is the
    autotuner's choice on a calibration subset."""
    pop = build_population(args.count)
    import torch
    import gapgb
    import gapgb.synth as S
    from gapgb import tune
    dev = torch.device("cuda", 0)
    off, sp, lat, pos = pop
    Sn, N = len(off) - 1, int(off[-1])
    ty, al, rc, ze = S.sf_table()
    zt = np.array([3, 8, 14, 26], np.int32)
    wt = zt.astype(np.float64)
    D = 2 * len(ty)
    probe = gapgb.GapModel.create(zt, wt, ty, al, rc, np.ones(D), np.zeros((1, D)), np.zeros(1),
                                  sf_zeta=ze)
    sub = int(off[40])
    X = probe.descriptors(off[:41], sp[:sub], lat[:40], pos[:sub])
    probe.close()
    theta, mm, coeff = S.model_arrays(X, M_SPARSE, theta_scale=1.0, coeff_std=1e-3, seed=0)
    m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    # calibration subset: the first 160 cells (about 21 k atoms, above the
    # library's two-pipeline threshold, so that knob is timed too)
    ncal = 160
    cal = int(off[ncal])
    best = tune.autotune(m, off[:ncal + 1], sp[:cal], lat[:ncal], pos[:cal], reps=3)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in (("off", off), ("sp", sp), ("lat", lat), ("pos", pos))}
    E = torch.zeros(Sn, dtype=torch.float64, device=dev)
    F = torch.zeros(N, 3, dtype=torch.float64, device=dev)
    St = torch.zeros(Sn, 6, dtype=torch.float64, device=dev)
    # the tuned capacity covers the calibration subset; the population may need more
    m.set_neighbour_cap(max(int(best["cap"]), 128))
    g = m.graph(Sn, N, int(np.diff(off).max()), t["off"].data_ptr(), t["sp"].data_ptr(),
                t["lat"].data_ptr(), t["pos"].data_ptr(), 1, E.data_ptr(), F.data_ptr(),
                St.data_ptr())
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        g.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    m.check_device_status()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    stop, lines = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, lines), daemon=True)
    th.start()
    time.sleep(0.3)
    for a, b in evs:
        flush.zero_()
        a.record(stream)
        g.launch(stream.cuda_stream)
        b.record(stream)
    torch.cuda.synchronize()
    stop.set()
    th.join()
    m.check_device_status()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    g.close()

    # end to end through the host-buffer call: pinned host inputs and outputs,
    # both copies inside the timed region
    h = {k: v.cpu().pin_memory() for k, v in t.items()}
    hE = torch.zeros(Sn, dtype=torch.float64).pin_memory()
    hF = torch.zeros(N, 3, dtype=torch.float64).pin_memory()
    hS = torch.zeros(Sn, 6, dtype=torch.float64).pin_memory()

    def host_step():
        m.eval_batch_host_ptrs(Sn, h["off"].data_ptr(), h["sp"].data_ptr(), h["lat"].data_ptr(),
                               h["pos"].data_ptr(), 1, hE.data_ptr(), hF.data_ptr(),
                               hS.data_ptr())

    for _ in range(args.warmup):
        host_step()
    t_host = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_step()
        t_host += time.perf_counter() - t0
    e2e_s = t_host / args.steps
    assert np.allclose(hE.numpy(), E.cpu().numpy(), rtol=0, atol=1e-9 * max(1.0, float(np.abs(E.cpu().numpy()).max())))
    h2d = sum(v.numel() * v.element_size() for v in h.values())
    d2h = (hE.numel() + hF.numel() + hS.numel()) * 8

    # per-stage device times of the tuned configuration (library CUDA events)
    os.environ["GAPGB_PROFILE_STAGES"] = "1"
    prof = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    tune._apply(prof, best)
    prof.set_neighbour_cap(max(int(best["cap"]), 128))
    stages = np.zeros(4)
    maxa = int(np.diff(off).max())
    for it in range(args.warmup + 3):
        flush.zero_()
        prof.eval_batch_ptrs(Sn, N, maxa, t["off"].data_ptr(), t["sp"].data_ptr(),
                             t["lat"].data_ptr(), t["pos"].data_ptr(), 1, E.data_ptr(),
                             F.data_ptr(), St.data_ptr(), 0, stream.cuda_stream)
        prof.check_device_status()
        if it >= args.warmup:
            stages += np.array(prof.stage_times())
    stages /= 3
    # slots and contributing angular pairs per atom on 64 of the cells (the
    # library's own neighbour list), for the per-atom byte and flop counts
    P, T = population_pair_stats(prof, pop, 64, float(rc.max()))
    prof.close()
    os.environ["GAPGB_PROFILE_STAGES"] = "0"
    roof = roofline(stages, N, D, best["precision"], simt=gapgb.measure_peaks(), P=P, T=T,
                    traffic_file=False,
                    tf32_tflops=measure_tf32_tflops() if best["precision"] == "tf32" else None)
    roof["slots_per_atom"], roof["pairs_per_atom"] = P, T

    line = {"metric": METRIC, "value": N / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": best["precision"], "data": "synthetic",
            "config": {"workload": "population%d" % Sn, "atoms": N,
                       "structures": Sn, "graph": "one CUDA graph launch per step",
                       "autotuned": {k: best.get(k) for k in ("precision", "generic_kernels", "cap",
                                                              "pipelines")},
                       "tune_errors": {"dE_per_atom": best["dE_per_atom"], "dF": best["dF"]},
                       "l2": "flushed between steps (512 MB write)"},
            "e2e": {"value": N / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "call": "gapgb_eval_batch (host buffers)"},
            "roofline": roof,
            # one graph launch per step holding the 10 kernels of a grouped-kernel
            # evaluation (see the headline workload's count); the generic
            # kernels add the reverse slots, the force gather and the orphans
            "gpu_launches": step_kernels(best["precision"], N, bool(best["generic_kernels"]),
                                         int(best.get("pipelines", 2))) * args.steps,
            "clocks": summarize_clocks(lines)}
    m.close()
    line["cpu_baseline"] = population_cpu_baseline(
        (zt, wt, ty, al, rc, ze, theta, mm, coeff), pop, 256)
    print(json.dumps(line), flush=True)


def population_pair_stats(model, pop, count, rc):
    """Mean slots and contributing angular pairs (j < k, r_ij, r_ik, r_jk <= rc)
    per atom over the first `count` cells of a population."""
    off, sp, lat, pos = pop
    slots = pairs = atoms = 0
    for s in range(count):
        a, b = int(off[s]), int(off[s + 1])
        cnt, nb = model.neighbors(sp[a:b], lat[s], pos[a:b], cap=400)
        for i in range(b - a):
            # rows (x, y, z, r, w, j + 1): the image position and its distance
            v = nb[i, :cnt[i], :3][nb[i, :cnt[i], 3] <= rc]
            d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=-1)
            pairs += int(np.triu(d <= rc, 1).sum())
            slots += int(cnt[i])
        atoms += b - a
    return slots / atoms, pairs / atoms


def population_cpu_baseline(arrays, pop, count):
    """The oracle on all host cores over the first `count` cells of the
    population (a bounded sample of the same workload)."""
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import write_model_file
    from oracle import oracle
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    off, sp, lat, pos = pop
    cores = len(os.sched_getaffinity(0))
    n = int(off[count])
    with tempfile.TemporaryDirectory() as d:
        om = oracle.Model(write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta, mm,
                                           coeff, ze))
        t0 = time.perf_counter()
        oracle.gap_calc_batch(om, off[:count + 1], sp[:n], lat[:count], pos[:n], 6.0, cores)
        dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "the first %d population cells (%d atoms) on %d host threads, %.1f s"
                      % (count, n, cores, dt)}


def nn_distances(lat, pos):
    """Nearest-neighbour distance of every atom of one cell (minimum image;
    the cell is at least twice as wide as the distances of interest)."""
    inv = np.linalg.inv(lat)
    f = pos @ inv
    d = f[:, None, :] - f[None, :, :]
    d -= np.round(d)
    r = np.sqrt(((d @ lat) ** 2).sum(-1))
    np.fill_diagonal(r, np.inf)
    return r.min(1)


def _alloy_chunk(args):
    seed0, count = args
    import gapgb.synth as S
    return S.pack([S.alloy512(seed=seed0 + s) for s in range(count)])


def build_alloy_set(count, seed0, workers=None):
    """`count` seeded alloy512 cells (seeds seed0 ..), packed, generated by a
    spawn-started process pool."""
    import multiprocessing as mp
    workers = workers or max(1, min(16, len(os.sched_getaffinity(0))))
    chunk = (count + workers - 1) // workers
    jobs = [(seed0 + w * chunk, min(chunk, count - w * chunk)) for w in range(workers)
            if count - w * chunk > 0]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_alloy_chunk, jobs)
    offs, sps, lats, poss = [], [], [], []
    base = 0
    for off, sp, lat, pos in parts:
        offs.append(off[:-1] + base)
        base += int(off[-1])
        sps.append(sp), lats.append(lat), poss.append(pos)
    off = np.concatenate(offs + [np.array([base])]).astype(np.int32)
    return off, np.concatenate(sps), np.concatenate(lats), np.concatenate(poss)


def run_surrogate(args):
    """The learned surrogate with GPR fallback (ternary alloy cells, the smooth
    alloy GAP: M = 4000, theta = 4 std).  Labels: the tensor-core GPR path on
    `train_structs` seeded cells; training: the library's own kernels; timed:
    the surrogate-with-fallback evaluation of `count` held-out cells in chunks
    of 512 cells (device buffers, CUDA events), beside the plain FP64 path and
    the tensor-core GPR path on the same chunks.  Errors are against the FP64
    path on every held-out atom and against the CPU oracle on two cells."""
    train_set = build_alloy_set(args.train_structs, 1_000_000)
    held = build_alloy_set(args.count, 9_000_000)
    import torch
    import gapgb
    import gapgb.synth as S
    import gapgb.surrogate as SU
    dev = torch.device("cuda", 0)
    arrays = S.alloy_model(M=M_SPARSE, theta_scale=args.surrogate_theta, coeff_std=1e-3, seed=0,
                           ncells=8)
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays

    def new_model(prec):
        m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
        m.set_neighbour_cap(96)
        m.set_precision(prec)
        return m

    # labels and training
    t0 = time.perf_counter()
    lab = new_model("tc")
    off, sp, lat, pos = train_set
    G, e, t = SU.gpr_labels(lab, off, sp, lat, pos)
    lab.close()
    torch.cuda.synchronize()
    t_label = time.perf_counter() - t0
    Zd = torch.from_numpy(sp).to(dev)
    sur = SU.Surrogate(zt, G.shape[1], 128, 4, seed=0)
    SU.fit_norm(sur, G, e, Zd)
    t0 = time.perf_counter()
    hist = SU.train(sur, G, e, t, Zd, epochs=args.epochs, rows_per_species=1024, lam=1.0,
                    lr=2e-3, lr_final=2e-5, seed=0)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    n_train = int(off[-1])
    # the contact radius of the force-sensitive trigger, from the training
    # cells alone: a low quantile of their atoms' nearest-neighbour distances
    contact = args.contact
    if contact is None:
        nn = np.concatenate([nn_distances(lat[s_], pos[off[s_]:off[s_ + 1]])
                             for s_ in range(min(400, len(off) - 1))])
        contact = float(np.quantile(nn, 0.002))
    # the gradient-spread trigger, calibrated on training atoms: quantiles of
    # the members' dE/dG spread (the chosen one flags about 1 % of them)
    gs = SU.grad_spread(sur, G[:1 << 20], Zd[:1 << 20]).double().cpu().numpy()
    gq = {q: float(np.quantile(gs, q)) for q in (0.9, 0.97, 0.99, 0.997)}
    gspread = gq[0.99]
    del G, e, t, Zd
    torch.cuda.empty_cache()

    # held-out evaluation in chunks of 512 cells
    off, sp, lat, pos = held
    Sh, Nh = len(off) - 1, int(off[-1])
    CH = 512
    chunks = []
    for c0 in range(0, Sh, CH):
        c1 = min(Sh, c0 + CH)
        a0, a1 = int(off[c0]), int(off[c1])
        chunks.append(dict(S=c1 - c0, N=a1 - a0, a0=a0, c0=c0,
                           off=torch.from_numpy(off[c0:c1 + 1] - a0).to(dev),
                           sp=torch.from_numpy(sp[a0:a1]).to(dev),
                           lat=torch.from_numpy(np.ascontiguousarray(lat[c0:c1])).to(dev),
                           pos=torch.from_numpy(np.ascontiguousarray(pos[a0:a1])).to(dev)))
    nmax = max(c["N"] for c in chunks)
    smax = max(c["S"] for c in chunks)
    d_E = torch.zeros(smax, dtype=torch.float64, device=dev)
    d_F = torch.zeros(nmax, 3, dtype=torch.float64, device=dev)
    d_St = torch.zeros(smax, 6, dtype=torch.float64, device=dev)
    d_ae = torch.zeros(nmax, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def step(m, c):
        m.eval_batch_ptrs(c["S"], c["N"], ATOMS, c["off"].data_ptr(), c["sp"].data_ptr(),
                          c["lat"].data_ptr(), c["pos"].data_ptr(), 1, d_E.data_ptr(),
                          d_F.data_ptr(), d_St.data_ptr(), d_ae.data_ptr(), stream.cuda_stream)

    def timed(m, cs, sampler=False):
        for _ in range(max(3, args.warmup)):
            step(m, cs[0])
        torch.cuda.synchronize()
        m.check_device_status()
        stop, lines, th = threading.Event(), [], None
        if sampler:
            th = threading.Thread(target=clocks_sampler, args=(stop, lines), daemon=True)
            th.start()
            time.sleep(0.3)
        evs = []
        for c in cs:
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step(m, c)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        if th:
            stop.set()
            th.join()
        m.check_device_status()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        return sum(c["N"] for c in cs) / (ms * 1e-3), ms, summarize_clocks(lines)

    def outputs(m, cs):
        ae, F, E = [], [], []
        for c in cs:
            step(m, c)
            torch.cuda.synchronize()
            m.check_device_status()
            ae.append(d_ae[:c["N"]].cpu().numpy().copy())
            F.append(d_F[:c["N"]].cpu().numpy().copy())
            E.append(d_E[:c["S"]].cpu().numpy().copy())
        return np.concatenate(ae), np.concatenate(F), np.concatenate(E)

    m_p = new_model("fp64")
    ae_p, F_p, E_p = outputs(m_p, chunks)

    def with_fallback(m, thr, con, gsp=0.0):
        m.attach_surrogate(sur, threshold=thr, contact=con, grad_spread=gsp)
        m.set_precision("surrogate")
        ae, F, E = [], [], []
        nfb = 0
        for c in chunks:
            step(m, c)
            torch.cuda.synchronize()
            m.check_device_status()
            nfb += m.fallback_count()
            ae.append(d_ae[:c["N"]].cpu().numpy().copy())
            F.append(d_F[:c["N"]].cpu().numpy().copy())
            E.append(d_E[:c["S"]].cpu().numpy().copy())
        return np.concatenate(ae), np.concatenate(F), np.concatenate(E), nfb

    # fallback fraction against the largest errors, over committee thresholds
    # and contact radii (the chosen configuration is the last entry)
    m_s = new_model("mixed")
    sweep = []
    configs = [(args.threshold, 0.0, 0.0), (0.001, 0.0, 0.0), (0.0002, 0.0, 0.0),
               (args.threshold, contact, 0.0), (args.threshold, contact + 0.1, 0.0)]
    configs += [(args.threshold, 0.0, gq[q]) for q in sorted(gq)]
    configs += [(args.threshold, contact, gq[q]) for q in sorted(gq)]
    for thr, con, gsp in configs:
        ae_x, F_x, _, nfb_x = with_fallback(m_s, thr, con, gsp)
        sweep.append({"threshold_eV": thr, "contact_A": con, "grad_spread": gsp,
                      "fallback_fraction": nfb_x / Nh,
                      "F_max": float(np.abs(F_x - F_p).max()),
                      "F_p999": float(np.quantile(np.abs(F_x - F_p), 0.999)),
                      "e_atom_max": float(np.abs(ae_x - ae_p).max())})
    # timed: the committee and contact triggers (the configuration whose
    # fallback stays cheap); beside it the gradient-spread trigger added,
    # whose extra fallback atoms run through the FP64 GPR
    ae_g, F_g, _, nfb_g = with_fallback(m_s, args.threshold, contact, gspread)
    value_g, _, _ = timed(m_s, chunks)
    ae_s, F_s, E_s, nfb = with_fallback(m_s, args.threshold, contact, 0.0)
    value, ms_total, clocks = timed(m_s, chunks, sampler=True)
    # stage times of the surrogate form on one chunk
    os.environ["GAPGB_PROFILE_STAGES"] = "1"
    prof = new_model("mixed")
    prof.attach_surrogate(sur, threshold=args.threshold, contact=contact)
    prof.set_precision("surrogate")
    stages = np.zeros(4)
    for it in range(6):
        flush.zero_()
        step(prof, chunks[0])
        prof.check_device_status()
        if it >= 3:
            stages += np.array(prof.stage_times())
    stages /= 3
    prof.close()
    os.environ["GAPGB_PROFILE_STAGES"] = "0"
    m_tc = new_model("tc")
    tc_value, _, _ = timed(m_tc, chunks)
    m_tc.close()
    plain_value, _, _ = timed(m_p, chunks[:2])
    m_p.close()
    de = ae_s - ae_p
    dF = F_s - F_p
    dE = (E_s - E_p) / np.diff(off)
    # two held-out cells against the CPU oracle (FP64 restatement of the reference)
    oracle_err = None
    try:
        import tempfile
        from oracle import oracle
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from helpers import write_model_file
        oracle.build()
        with tempfile.TemporaryDirectory() as d:
            om = oracle.Model(write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta,
                                               mm, coeff, ze))
            errs = []
            for s in range(2):
                a0, a1 = int(off[s]), int(off[s + 1])
                eo, fo, _, _ = oracle.gap_calc(om, sp[a0:a1], lat[s], pos[a0:a1], 6.0, True)
                errs.append((abs(E_s[s] - eo) / (a1 - a0), float(np.abs(F_s[a0:a1] - fo).max())))
            oracle_err = {"dE_per_atom_max": max(x[0] for x in errs),
                          "dF_max": max(x[1] for x in errs), "structures": 2}
    except Exception as ex:  # the oracle is test infrastructure; its absence does not stop the bench
        oracle_err = {"unavailable": str(ex)[:200]}
    # kernels per surrogate evaluation: prep x2, neighbours, descriptors,
    # surrogate (count, segments, scatter, weight image, row image, tensor-core
    # MLP, committee), fallback select, row-list GPR + reduce, slot gradients
    # (forces scattered in the same kernel), structure partial + final sums
    launches_per_eval = 17
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
            "steps": len(chunks), "warmup": max(3, args.warmup),
            "ms_per_step": ms_total / len(chunks), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16/f32 surrogate + f64 GPR fallback",
            "data": "synthetic",
            "config": {"workload": "surrogate: %d held-out alloy512 cells" % Sh,
                       "atoms": Nh, "step": "one chunk of %d cells" % CH,
                       "model": "alloy GAP M=4000 theta=%g std, D=64" % args.surrogate_theta,
                       "network": "per-species 64-128-128-1 SiLU, 4-member committee",
                       "threshold_eV": args.threshold, "contact_A": contact,
                       "grad_spread_training_quantiles": {str(k): v for k, v in gq.items()},
                       "l2": "flushed between steps (512 MB write)"},
            "train": {"structures": args.train_structs, "atoms": n_train, "epochs": args.epochs,
                      "rows_per_species": 1024, "label_s": t_label, "train_s": t_train,
                      "loss_first_last": [hist[0], hist[-1]]},
            "fallback": {"atoms": int(nfb), "fraction": nfb / Nh,
                         "trigger": "committee std > threshold, or a neighbour closer than "
                                    "contact_A (0.2% quantile of the training cells' "
                                    "nearest-neighbour distances)"},
            "with_grad_spread": {"grad_spread": gspread, "quantile": 0.99, "value": value_g,
                                 "unit": UNIT, "fallback_fraction": nfb_g / Nh,
                                 "F_max": float(np.abs(F_g - F_p).max()),
                                 "F_p999": float(np.quantile(np.abs(F_g - F_p), 0.999))},
            "fallback_sweep": sweep,
            "errors_vs_fp64": {"e_atom_rms": float(np.sqrt(np.mean(de ** 2))),
                               "e_atom_p999": float(np.quantile(np.abs(de), 0.999)),
                               "e_atom_max": float(np.abs(de).max()),
                               "F_p999": float(np.quantile(np.abs(dF), 0.999)),
                               "E_per_atom_max": float(np.abs(dE).max()),
                               "F_rms": float(np.sqrt(np.mean(dF ** 2))),
                               "F_max": float(np.abs(dF).max()), "atoms": Nh},
            "errors_vs_oracle": oracle_err,
            "plain_fp64": {"value": plain_value, "unit": UNIT},
            "tc_gpr": {"value": tc_value, "unit": UNIT},
            "speedup_vs_plain": value / plain_value,
            "stage_ms_chunk": {"neighbours": stages[0], "descriptors": stages[1],
                               "surrogate_and_fallback": stages[2], "chain_rule": stages[3]},
            "gpu_launches": launches_per_eval * len(chunks),
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    m_s.close()
    sur.close()


def run_md(args):
    """MD workload: 32768-atom Si/Ge (50/50) diamond cell, a = 5.54 A, jitter
    0.1 A; GAP with M = 8000 sparse points (library descriptors of a second
    seeded cell, theta = 1 std, coeff ~ N(0, 1e-3)); Maxwell-Boltzmann
    velocities at 600 K; NVE velocity Verlet, dt = 1 fs, neighbour rebuild
    (skin 0.5 A) every 10 steps, each step one graph launch.  The tensor-core
    form and the plain FP64 path run the same trajectory start; reported:
    atom-steps/s of each, NVE energy drift, and force / stress differences on
    identical configurations (t = 0 and the FP64 run's last step)."""
    import torch
    import gapgb
    import gapgb.synth as S
    from gapgb.md import MD, masses_of, maxwell_boltzmann
    L = gapgb.load()
    dev = torch.device("cuda", 0)
    lat, pos, z = S.sige(seed=0, reps=args.md_reps)
    arrays = S.model_from_cells([S.sige(seed=1, reps=args.md_reps)], [14, 32], 8000,
                                theta_scale=1.0, coeff_std=1e-3, seed=0)
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    N = len(z)
    masses = masses_of(z)
    vel = maxwell_boltzmann([0, N], masses, 600.0, seed=0)
    # a dedicated stream: the MD steps and the timing events share it (a null
    # handle would select the MD object's own stream instead)
    stream = torch.cuda.Stream(dev)
    res = {}
    for prec in ("tc", "fp64"):
        m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
        m.set_precision(prec)
        m.set_neighbour_cap(64)
        md = MD(m, [0, N], z, lat[None], pos, vel, masses, dt=1.0, skin=0.5, rebuild_every=10)
        E0, F0, S0, K0 = md.outputs()
        ep = torch.zeros((args.md_steps, 1), dtype=torch.float64, device=dev)
        ek = torch.zeros((args.md_steps, 1), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stop, lines, th = threading.Event(), [], None
        if prec == "tc":
            th = threading.Thread(target=clocks_sampler, args=(stop, lines), daemon=True)
            th.start()
            time.sleep(0.3)
        a.record(stream)
        st = L.gapgb_md_run(md.handle, args.md_steps, ep.data_ptr(), ek.data_ptr(),
                            stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        if th:
            stop.set()
            th.join()
        if st != 0:
            raise gapgb.GapError(st, "gapgb_md_run")
        md.check()
        ms = a.elapsed_time(b)
        et = (ep + ek).cpu().numpy()[:, 0]
        e_init = E0[0] + K0[0]
        res[prec] = dict(ms=ms, value=N * args.md_steps / (ms * 1e-3), E0=E0, F0=F0, S0=S0,
                         drift=float(np.abs(et - e_init).max() / N),
                         drift_end=float((et[-1] - e_init) / N),
                         final=md.positions(), out=md.outputs(), clocks=summarize_clocks(lines))
        md.close()
        m.close()
    # the FP64 run's last configuration evaluated in the tensor-core form
    m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    m.set_precision("tc")
    Et, Ft, St = m.eval_batch([0, N], z, lat[None], res["fp64"]["final"])
    m.close()
    Ep, Fp, Sp, _ = res["fp64"]["out"]
    tc, fp = res["tc"], res["fp64"]
    line = {"metric": METRIC, "value": tc["value"], "unit": "atom-steps/s", "n_gpus": 1,
            "steps": args.md_steps, "warmup": 0, "ms_per_step": tc["ms"] / args.md_steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3/f32 (tensor-core form)", "data": "synthetic",
            "config": {"workload": "md: Si/Ge 50/50 diamond %d^3 (%d atoms), a=5.54, jitter 0.1"
                                   % (args.md_reps, N),
                       "model": "M=8000, D=64, theta=1 std", "integrator":
                       "NVE velocity Verlet dt=1 fs, 600 K MB start, rebuild every 10 (skin 0.5 A)",
                       "step": "one CUDA graph launch"},
            "plain_fp64": {"value": fp["value"], "unit": "atom-steps/s",
                           "ms_per_step": fp["ms"] / args.md_steps},
            "speedup_vs_plain": tc["value"] / fp["value"],
            "nve_drift_per_atom_eV": {"tc_max": tc["drift"], "fp64_max": fp["drift"],
                                      "tc_end": tc["drift_end"], "fp64_end": fp["drift_end"]},
            "tc_vs_fp64_same_config": {
                "t0": {"dE_per_atom": float(abs(tc["E0"][0] - fp["E0"][0]) / N),
                       "dF_max": float(np.abs(tc["F0"] - fp["F0"]).max()),
                       "dF_rms": float(np.sqrt(np.mean((tc["F0"] - fp["F0"]) ** 2))),
                       "dstress_max_GPa": float(np.abs(tc["S0"] - fp["S0"]).max())},
                "t_end": {"dE_per_atom": float(abs(Et[0] - Ep[0]) / N),
                          "dF_max": float(np.abs(Ft - Fp).max()),
                          "dstress_max_GPa": float(np.abs(St - Sp).max())}},
            # per step: kick+drift, wrap or skin check, prep x2, refresh,
            # descriptors, tensor-core GPR (prep + kernel), slot gradients with
            # the force scatter, structure sums x2, kick, kinetic sums x2 = 14,
            # plus 4 for the second pipeline of a large batch; a rebuild step
            # adds the build, the bins (offsets, count, scan, fill) and the
            # binned build in place of the refresh (+5)
            "gpu_launches": (14 + step_kernels("tc", N) - 9) * args.md_steps
                            + 5 * (args.md_steps // 10),
            "clocks": tc["clocks"]}
    print(json.dumps(line), flush=True)


def run_precision(args):
    """Precision-form comparison: the alloy step (512-atom cells, the default
    batch as in the headline workload, M = 4000,
    D = 64) in every arithmetic form of the contraction - FP64 (plain), FP32
    SIMT, mixed (FP32 descriptors, FP64 GPR), TF32 tensor cores, split-BF16x3
    tensor cores - each timed on device-resident inputs (CUDA events, L2
    flushed) with its error against the FP64 path on every atom and against
    the CPU oracle on one cell."""
    import torch
    import gapgb
    dev = torch.device("cuda", 0)
    arrays = make_model()
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    structs, (off, sp, lat, pos) = workload(0, default_batch(args, dev))
    S, N = len(structs), int(off[-1])
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in (("off", off), ("sp", sp), ("lat", lat), ("pos", pos))}
    E = torch.zeros(S, dtype=torch.float64, device=dev)
    F = torch.zeros(N, 3, dtype=torch.float64, device=dev)
    St = torch.zeros(S, 6, dtype=torch.float64, device=dev)
    AE = torch.zeros(N, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    res, outs = {}, {}
    for prec in ("fp64", "fp32", "mixed", "tf32", "tc"):
        m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
        m.set_precision(prec)
        m.set_neighbour_cap(96)

        def step():
            m.eval_batch_ptrs(S, N, ATOMS, t["off"].data_ptr(), t["sp"].data_ptr(),
                              t["lat"].data_ptr(), t["pos"].data_ptr(), 1, E.data_ptr(),
                              F.data_ptr(), St.data_ptr(), AE.data_ptr(), stream.cuda_stream)
        steps = 2 if prec in ("fp64", "mixed") else args.steps
        for _ in range(max(3, args.warmup) if steps > 2 else 1):
            step()
        torch.cuda.synchronize()
        m.check_device_status()
        evs = []
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        m.check_device_status()
        ms = sum(a.elapsed_time(b) for a, b in evs) / steps
        outs[prec] = (AE.cpu().numpy().copy(), F.cpu().numpy().copy(), St.cpu().numpy().copy(),
                      E.cpu().numpy().copy())
        res[prec] = {"atoms_per_s": N / (ms * 1e-3), "ms_per_step": ms}
        m.close()
    ae0, f0, s0, e0 = outs["fp64"]
    for prec in res:
        ae, f, st, e = outs[prec]
        res[prec]["vs_fp64_path"] = {"dE_per_atom_max": float(np.abs(e - e0).max() / ATOMS),
                                     "de_atom_max": float(np.abs(ae - ae0).max()),
                                     "dF_max": float(np.abs(f - f0).max()),
                                     "dstress_max_GPa": float(np.abs(st - s0).max())}
    orc = None if args.no_oracle else oracle_errors(
        arrays, structs, {k: (v[3], v[1], v[2]) for k, v in outs.items()})
    line = {"metric": METRIC, "value": res["tc"]["atoms_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["tc"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3/f32", "data": "synthetic",
            "config": {"workload": "precision forms on alloy512 x %d (D=64, M=4000)" % S,
                       "atoms": N, "l2": "flushed between steps (512 MB write)"},
            "forms": res, "errors_vs_oracle": orc,
            "gpu_launches": step_kernels("tc", N) * args.steps}
    print(json.dumps(line), flush=True)


def qmm_of(mm, theta, lam=1e-2):
    """(K_MM + lam I)^-1 of a model's sparse points (the inverse covariance a
    fitting code would hand over as qmm)."""
    X = mm / theta
    n2 = (X * X).sum(1)
    d2 = np.maximum(n2[:, None] + n2[None, :] - 2.0 * (X @ X.T), 0.0)
    return np.linalg.inv(np.exp(-0.5 * d2) + lam * np.eye(len(mm)))


def run_variance(args):
    """The GPR variance block (gap_calc.f90:206-210, commented out in the
    reference) on the alloy workload: 64 alloy512 cells (32768 atoms),
    M = 4000, D = 64, qmm = (K_MM + 0.01 I)^-1 of the model's sparse points.
    The tensor-core form (FP32 K, split-BF16x3 products, FP32 accumulation)
    is timed through gapgb_variance with host buffers (e2e) and its kernels
    alone with device events; the FP64 form runs once for the comparison on
    every atom, and the CPU oracle on one cell."""
    os.environ["GAPGB_PROFILE_STAGES"] = "1"  # read at the model's device upload
    import gapgb
    arrays = make_model()
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    Q = qmm_of(mm, theta)
    structs, (off, sp, lat, pos) = workload(0, args.batch or 64)
    S, N, M = len(structs), int(off[-1]), len(mm)
    m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    m.set_qmm(Q)
    m.set_precision("tc")
    m.set_neighbour_cap(96)
    for _ in range(max(3, args.warmup)):
        m.variance(off, sp, lat, pos)
    stop, lines = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, lines), daemon=True)
    th.start()
    time.sleep(0.3)
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        covf, var = m.variance(off, sp, lat, pos)
        wall.append(time.perf_counter() - t0)
        kern.append(m.variance_time())
    stop.set()
    th.join()
    m.set_precision("fp64")
    t0 = time.perf_counter()
    c64, v64 = m.variance(off, sp, lat, pos)
    t64 = time.perf_counter() - t0
    k64 = m.variance_time()
    m.close()
    kms = sum(kern) / len(kern)
    wms = 1e3 * sum(wall) / len(wall)
    peaks, src = load_peaks()
    peak = peaks["bf16_tflops"]
    Mp = (M + 255) // 256 * 256
    flops = 2.0 * N * M * M  # the contraction K qmm^T, once
    mma = 3 * 2.0 * ((N + 127) // 128 * 128) * Mp * Mp  # three split products, padded
    achieved = flops / (kms * 1e-3) / 1e12
    orc = None
    if not args.no_oracle:
        from oracle import oracle
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import tempfile
        from helpers import write_model_file
        with tempfile.TemporaryDirectory() as d:
            om = oracle.Model(write_model_file(os.path.join(d, "gp"), zt, wt, ty, al, rc, theta,
                                               mm, coeff, ze))
            l0, p0, z0 = structs[0]
            *_, ex = oracle.gap_calc(om, z0, l0, p0, 6.0, False, extras=True)
            oc, ov = oracle.variance(om, ex["xx"], Q)
        n0 = len(p0)
        orc = {"tc_dcovf_max": float(np.abs(covf[:n0] - oc).max()),
               "fp64_dcovf_max": float(np.abs(c64[:n0] - oc).max()),
               "tc_dvariance": float(abs(var[0] - ov)), "atoms": n0}
    line = {"metric": "atom variance evals/s", "value": N / (kms * 1e-3), "unit": "atoms/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": kms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3/f32 (tensor-core form)", "data": "synthetic",
            "config": {"workload": "variance: alloy512 x %d (%d atoms), M=%d, D=64, "
                                   "qmm=(K_MM+0.01 I)^-1" % (S, N, M),
                       "l2": "inputs larger than L2 (K tiles %d MB)" % (N * Mp * 4 >> 20)},
            "e2e": {"value": N / (wms * 1e-3), "unit": "atoms/s", "ms_per_call": wms,
                    "h2d_bytes_per_step": int(off.nbytes + sp.nbytes + lat.nbytes + pos.nbytes),
                    "d2h_bytes_per_step": int(covf.nbytes + var.nbytes),
                    "note": "gapgb_variance: neighbour list, descriptors and the variance"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak,
                         "peak_source": src + " bf16_tflops",
                         "traffic": None, "mma_tflops": mma / (kms * 1e-3) / 1e12,
                         "note": "achieved counts 2*N*M^2 (the contraction once); mma_tflops the "
                                 "three split-BF16 products issued on padded tiles"},
            "fp64_form": {"value": N / (k64 * 1e-3), "unit": "atoms/s", "kernel_ms": k64,
                          "call_ms": 1e3 * t64},
            "speedup_vs_fp64_form": k64 / kms,
            "tc_vs_fp64_form": {"dcovf_max": float(np.abs(covf - c64).max()),
                                "dcovf_mean": float(np.abs(covf - c64).mean()),
                                "dvariance_max": float(np.abs(var - v64).max()),
                                "covf_range": [float(c64.min()), float(c64.max())]},
            "errors_vs_oracle": orc,
            # per call: prep x2, neighbour build, reverse, descriptors, centring,
            # K tiles, contraction, row sums, structure means
            "gpu_launches": 10 * args.steps,
            "clocks": summarize_clocks(lines)}
    print(json.dumps(line), flush=True)


def run_fit(args):
    """Sparse-GPR fitting on the device (gapgb_fit_energies): the alloy
    model's M = 4000 sparse points, teacher energies from the model itself
    (FP64 path) on --fit-structs alloy512 cells, refitted from those energies
    (sigma_e = 1 meV/atom, jitter 1e-6); reported: the fit's wall time per
    call, training atoms per second, the refit's training RMSE and its
    held-out RMSE against the teacher on 16 further cells."""
    import gapgb
    import gapgb.synth as S
    arrays = make_model()
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays
    ns = args.fit_structs
    off, sp, lat, pos = S.pack([S.alloy512(seed=2000 + s) for s in range(ns)])
    N = int(off[-1])
    n = np.diff(off)
    teacher = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
    teacher.set_precision("fp64")
    E, _, _ = teacher.eval_batch(off, sp, lat, pos, lgrad=False)
    offh, sph, lath, posh = S.pack([S.alloy512(seed=9000 + s) for s in range(16)])
    Eh_t, _, _ = teacher.eval_batch(offh, sph, lath, posh, lgrad=False)
    teacher.close()
    m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, np.zeros_like(coeff), sf_zeta=ze)
    m.set_precision("fp64")
    m.fit_energies(off, sp, lat, pos, E, sigma_e=1e-3, jitter=1e-6)  # warm-up
    times = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        c = m.fit_energies(off, sp, lat, pos, E, sigma_e=1e-3, jitter=1e-6)
        times.append(time.perf_counter() - t0)
    E2, _, _ = m.eval_batch(off, sp, lat, pos, lgrad=False)
    Eh, _, _ = m.eval_batch(offh, sph, lath, posh, lgrad=False)
    m.close()
    ms = 1e3 * sum(times) / len(times)
    line = {"metric": "training atoms fitted per second", "value": N / (ms * 1e-3),
            "unit": "atoms/s", "n_gpus": 1, "steps": len(times), "warmup": 1, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "fit: %d alloy512 cells (%d atoms), M=%d, D=64, sigma_e=1 meV/atom, "
                                   "jitter 1e-6" % (ns, N, len(mm)),
                       "step": "gapgb_fit_energies: FP64 descriptors, design rows, Gram, "
                               "Cholesky, solves"},
            "train_rmse_eV_per_atom": float(np.sqrt(np.mean(((E2 - E) / n) ** 2))),
            "heldout_rmse_eV_per_atom": float(np.sqrt(np.mean(((Eh - Eh_t) / 512) ** 2))),
            "teacher_energy_scale_eV_per_atom": float(np.abs(Eh_t / 512).max()),
            "coeff_max": float(np.abs(c).max()),
            # per call: prep x2, neighbour build, reverse, FP64 descriptors, K_MM, jitter,
            # weights, design rows, Gram, right-hand side, 3 per Cholesky panel (2 for the
            # last), solves
            "gpu_launches": (5 + 6 + 3 * ((len(mm) + 63) // 64) - 2 + 1) * len(times)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "fit" and args.impl != "reference":
        run_fit(args)
        return
    if args.workload == "variance" and args.impl != "reference":
        run_variance(args)
        return
    if args.workload == "precision" and args.impl != "reference":
        run_precision(args)
        return
    if args.workload == "md" and args.impl != "reference":
        run_md(args)
        return
    if args.workload == "population" and args.impl != "reference":
        run_population(args)
        return
    if args.workload == "surrogate" and args.impl != "reference":
        run_surrogate(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import gapgb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    os.environ.setdefault("GAPGB_PROFILE_STAGES", "0")
    dev = torch.device("cuda", local)
    arrays = make_model()
    zt, wt, ty, al, rc, ze, theta, mm, coeff = arrays

    def new_model(prec):
        m = gapgb.GapModel.create(zt, wt, ty, al, rc, theta, mm, coeff, sf_zeta=ze)
        m.set_precision(prec)
        m.set_neighbour_cap(96)
        m.set_pipelines(args.pipelines)
        return m

    structs, (off, sp, lat, pos) = workload(rank, default_batch(args, dev))
    S, N = len(structs), int(off[-1])
    d_off = torch.from_numpy(off).to(dev)
    d_sp = torch.from_numpy(sp).to(dev)
    d_lat = torch.from_numpy(lat).to(dev)
    d_pos = torch.from_numpy(pos).to(dev)
    d_E = torch.zeros(S, dtype=torch.float64, device=dev)
    d_F = torch.zeros(N, 3, dtype=torch.float64, device=dev)
    d_S = torch.zeros(S, 6, dtype=torch.float64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def device_step(m):
        m.eval_batch_ptrs(S, N, ATOMS, d_off.data_ptr(), d_sp.data_ptr(), d_lat.data_ptr(),
                          d_pos.data_ptr(), 1, d_E.data_ptr(), d_F.data_ptr(), d_S.data_ptr(),
                          0, stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def time_device(m, steps, warmup, sampler=None):
        for _ in range(warmup):
            device_step(m)
        torch.cuda.synchronize()
        m.check_device_status()
        barrier()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        stop, lines, th = threading.Event(), [], None
        if sampler:
            th = threading.Thread(target=clocks_sampler, args=(stop, lines), daemon=True)
            th.start()
            time.sleep(0.3)
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            device_step(m)
            b.record(stream)
        torch.cuda.synchronize()
        if th:
            stop.set()
            th.join()
        barrier()
        m.check_device_status()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        return max_over_ranks(ms, world, dev) / steps, summarize_clocks(lines)

    simt = gapgb.measure_peaks()  # the SIMT roofline denominators of this device
    chosen = new_model(args.precision)
    ms_step, clocks = time_device(chosen, args.steps, args.warmup, sampler=(rank == 0))
    value = world * N / (ms_step * 1e-3)
    res_chosen = (d_E.cpu().numpy().copy(), d_F.cpu().numpy().copy(), d_S.cpu().numpy().copy())
    gather = None
    if world > 1:
        # every structure's (E, F, stress) to rank 0: the job's only data
        # exchange, after the timed steps (the shards are the ranks' seed blocks)
        from gapgb import shard
        g_off = np.arange(world * S + 1, dtype=np.int64) * ATOMS
        shards = [np.arange(r * S, (r + 1) * S) for r in range(world)]
        barrier()
        t0 = time.perf_counter()
        got = shard.gather_results(d_E, d_F, d_S, g_off, shards, rank, device=dev)
        gather = {"ms": (time.perf_counter() - t0) * 1e3,
                  "bytes_per_rank": int(S * 7 * 8 + N * 3 * 8), "backend": "nccl all_gather"}
        if rank == 0:
            assert np.array_equal(got[0][:S], res_chosen[0])
            assert np.array_equal(got[1][:N], res_chosen[1])

    # per-stage device times (library CUDA events on the launch stream)
    os.environ["GAPGB_PROFILE_STAGES"] = "1"
    prof = new_model(args.precision)
    stages = np.zeros(4)
    for it in range(args.warmup + 3):
        flush.zero_()
        device_step(prof)
        prof.check_device_status()
        if it >= args.warmup:
            stages += np.array(prof.stage_times())
    stages /= 3
    prof.close()
    os.environ["GAPGB_PROFILE_STAGES"] = "0"

    # end to end through the host-buffer call, pinned host buffers
    h_off = torch.from_numpy(off).pin_memory()
    h_sp = torch.from_numpy(sp).pin_memory()
    h_lat = torch.from_numpy(lat).pin_memory()
    h_pos = torch.from_numpy(pos).pin_memory()
    h_E = torch.zeros(S, dtype=torch.float64).pin_memory()
    h_F = torch.zeros(N, 3, dtype=torch.float64).pin_memory()
    h_S = torch.zeros(S, 6, dtype=torch.float64).pin_memory()

    def host_step(m):
        m.eval_batch_host_ptrs(S, h_off.data_ptr(), h_sp.data_ptr(), h_lat.data_ptr(),
                               h_pos.data_ptr(), 1, h_E.data_ptr(), h_F.data_ptr(), h_S.data_ptr())

    for _ in range(args.warmup):
        host_step(chosen)
    barrier()
    t_host = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_step(chosen)
        t_host += time.perf_counter() - t0
    e2e_s = max_over_ranks(t_host / args.steps, world, dev)
    h2d = off.nbytes + sp.nbytes + lat.nbytes + pos.nbytes
    d2h = S * 8 + N * 3 * 8 + S * 6 * 8

    # plain FP64 path on the same workload
    plain = new_model("fp64")
    psteps = max(2, args.steps // 3)
    ms_plain, _ = time_device(plain, psteps, max(1, args.warmup // 2))
    res_plain = (d_E.cpu().numpy().copy(), d_F.cpu().numpy().copy(), d_S.cpu().numpy().copy())
    plain_value = world * N / (ms_plain * 1e-3)
    plain.close()
    # stage times of the plain FP64 path (two steps after one warm-up)
    os.environ["GAPGB_PROFILE_STAGES"] = "1"
    pprof = new_model("fp64")
    plain_stages = np.zeros(4)
    for it in range(3):
        flush.zero_()
        device_step(pprof)
        pprof.check_device_status()
        if it >= 1:
            plain_stages += np.array(pprof.stage_times())
    plain_stages /= 2
    pprof.close()
    os.environ["GAPGB_PROFILE_STAGES"] = "0"

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    errors = None if args.no_oracle else oracle_errors(
        arrays, structs, {"chosen": res_chosen, "plain": res_plain})

    roof = roofline(stages, N, 2 * len(ty), args.precision, simt=simt, plain_stages=plain_stages)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "tc": "bf16x3/f32", "tf32": "tf32/f32", "fp64": "f64",
                  "mixed": "f32/f64"}[args.precision],
        "data": "synthetic",
        "config": {"workload": "alloy512 ternary fcc (Z 13/28/40), D=64, M=4000",
                   "structures_per_step": S, "atoms_per_step_per_gpu": N,
                   "batch_rule": "one wave of the tensor-core GPR: 2 CTAs x 128 atoms per SM",
                   "precision": args.precision, "pipelines": args.pipelines,
                   "l2": "flushed between steps (512 MB write)"},
        "e2e": {"value": world * N / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "plain_fp64": {"value": plain_value, "unit": UNIT, "ms_per_step": ms_plain},
        "speedup_vs_plain": value / plain_value,
        "errors_vs_oracle": errors,
        "roofline": roof,
        "gpu_launches": None,
        "clocks": clocks,
    }
    if gather is not None:
        line["gather_to_rank0"] = gather
    # kernels launched per step (count from the library's launch sequence)
    line["gpu_launches"] = args.steps * step_kernels(args.precision, N, pipelines=args.pipelines)
    if world == 1:
        line["cpu_baseline"] = cpu_baseline(arrays)
        line["dropin_latency_ms"] = dropin_latency()
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
