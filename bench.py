#!/usr/bin/env python3
"""SGH hot-path benchmark: element-cycles/s of the plain FP64 RK2 SGH cycle on the
256^3 perturbed Sedov problem (16.8 M hexes, interior nodes jittered by
U(-0.1h, 0.1h) per axis from a seed, element and node ids randomly permuted,
gamma = 1.4, origin-corner energy 0.2467, CFL 0.4).  A step is one SGH cycle
(two RK stages) over the whole mesh.

Prints one JSON line.  Default: 1 GPU, 20 timed
cycles after 3 warm-up cycles.  Under torchrun (N > 1) every rank advances its own
replica (the path is run as independent replicas, no collective in the data
path); value = all ranks' element-cycles / max-over-ranks time.

  python bench.py [--steps K] [--warmup W] [--n 256] [--fp-mode exact|fma]
  python bench.py --impl reference     # the reference's own CPU SGH solver
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SGH element-cycles/s, 256^3 perturbed Sedov, FP64 RK2"
UNIT = "element-cycles/s"


def metric_of(args) -> str:
    """The headline metric; --problem noh measures the same quantity on the Noh
    implosion (every node moving from the first cycle)."""
    if getattr(args, "problem", "sedov") == "noh":
        return "SGH element-cycles/s, %d^3 perturbed Noh, FP64 RK2" % args.n
    return METRIC


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="elements per edge of the Sedov box")
    ap.add_argument("--problem", default="sedov", choices=["sedov", "noh"],
                    help="sedov (default): the blast from one corner element, the rest of the mesh at rest; "
                         "noh: the implosion, every node moving from the first cycle (the kernels do the "
                         "same work per element either way)")
    ap.add_argument("--fp-mode", default="fma", choices=["exact", "fma"],
                    help="fma (default): fused multiply-adds, within 1e-12 of the reference after one cycle "
                         "and 1e-9 after a full run on the gated fields; exact: the reference's arithmetic bit "
                         "for bit (also measured, as exact_mode, when the headline runs in fma)")
    ap.add_argument("--no-exact-leg", action="store_true")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-n", type=int, default=120, help="edge of the CPU baseline sample mesh")
    ap.add_argument("--cpu-cycles", type=int, default=6, help="timed cycles of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cpu-1thread", action="store_true",
                    help="skip the reference's one-thread figure on the CPU sample")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the parity leg (the GPU in both modes against the reference's own solver on the "
                         "CPU sample's deck, after one cycle and after K)")
    ap.add_argument("--no-batch-leg", action="store_true",
                    help="skip the batched-ensemble object of the default line")
    ap.add_argument("--no-adjoint-leg", action="store_true",
                    help="skip the discrete-adjoint object of the default line")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--batch", action="store_true",
                    help="run the batched-ensemble benchmark instead (instances/s vs looping the plain solver)")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--batch-cycles", type=int, default=100)
    ap.add_argument("--outputs", action="store_true",
                    help="graphics dumps: cycle time with the writer thread on vs off")
    ap.add_argument("--adjoint", action="store_true",
                    help="discrete adjoint: Sedov 64^3, 400 cycles, J = sum M (rho - rho_target)^2")
    ap.add_argument("--adj-n", type=int, default=64)
    ap.add_argument("--adj-cycles", type=int, default=400)
    ap.add_argument("--adj-ckpt", type=int, default=20)
    ap.add_argument("--adj-dirs", type=int, default=16)
    ap.add_argument("--strength", default=None, choices=["hypo", "hyper"],
                    help="strength-model run: the workload with the shipped hypo-elastic model as a hypo or "
                         "hyper model on every element, against the same problem without strength")
    ap.add_argument("--shear-modulus", type=float, default=1.0)
    ap.add_argument("--configs", action="store_true",
                    help="the small reference decks (Sedov 12^3 for 200 cycles, Noh 32^3 for 500) on the GPU "
                         "and on the reference CPU solver (all host cores and one)")
    ap.add_argument("--fp64-peak", action="store_true",
                    help="survey of the FP64 pipe: a pure fma/add/mul stream over chains per thread and "
                         "resident blocks (the roof the SGH kernels run at)")
    ap.add_argument("--rz", action="store_true",
                    help="2D-RZ run: jittered, permuted RZ Sedov on an n x n quad mesh (--rz-n)")
    ap.add_argument("--rz-n", type=int, default=4096)
    ap.add_argument("--rz-cpu-n", type=int, default=1024)
    return ap.parse_args(argv)


def workload(n: int, seed: int, problem: str = "sedov"):
    from fierro_gb300 import problems
    if problem == "noh":
        return problems.noh(n, length=1.0, jitter=0.1, seed=seed, permute=True, cycles=10 ** 9)
    return problems.sedov(n, length=1.2, energy=0.2467, gamma=1.4, jitter=0.1, seed=seed, permute=True,
                          cycles=10 ** 9)


def config_of(args, n=None):
    n = args.n if n is None else n
    common = {"elements": n ** 3, "nodes": (n + 1) ** 3, "rk_stages": 2, "seed": args.seed,
              "parallelism": "replicas" if args.gpus > 1 else "single",
              "l2": "inputs larger than L2 (device state > 10 GB vs 129 MB L2)"}
    if getattr(args, "problem", "sedov") == "noh":
        return dict({"workload": "noh3d_%d^3_jitter0.1_permuted" % n, "gamma": 5.0 / 3.0, "speed": -1.0,
                     "cfl": 0.3}, **common)
    return dict({"workload": "sedov3d_%d^3_jitter0.1_permuted" % n, "gamma": 1.4, "energy": 0.2467,
                 "cfl": 0.4}, **common)


# ------------------------------------------------------------------ distributed
def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 1
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    rank = int(os.environ.get("RANK", "0"))
    if backend == "nccl":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist.init_process_group(backend=backend)
    return dist, rank, world


def reduce_max(dist, value: float) -> float:
    """Max over ranks (the bench's time and the replicas' slowest rank)."""
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        # the CUDA device's UUID names the same GPU for nvidia-smi whatever
        # CUDA_VISIBLE_DEVICES renumbers; the index is the fallback
        self.index = str(index)
        try:
            import torch
            self.index = "GPU-" + str(torch.cuda.get_device_properties(index).uuid)
        except Exception:
            pass
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", self.index, "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ------------------------------------------------------------------ algorithmic bytes
def alg_bytes(kind: str, nn: int, ne: int, nnz: int) -> float:
    """Compulsory HBM bytes of one launch of each kernel: every array it touches
    counted once (FP64 state, int32 connectivity), gathers at perfect reuse."""
    if kind == "k_force":
        return ne * (32 + 192 + 5 * 8 + 4 + 4 + 192) + 4 * nnz + nn * 24
    if kind == "k_node":
        return nn * (4 + 8 + 1 + 48 + 72) + ne * (8 * 4 + 192)
    if kind == "k_elem":
        return ne * (32 + 192 + 8 + 8 + 8 + 16 + 5 * 8 + 192) + nn * 72
    return 0.0


# Per-element figures of the kernels from ncu captures of jittered Sedov (one
# kernel filter, three to six launches, --clock-control none).  FP64 thread
# instructions per element of one launch, exact and FMA modes, at 64^3.  DRAM
# bytes (dram__bytes_read + dram__bytes_write) per element of one launch at
# 128^3 (state 13x the L2), applied to 256^3 by the element count (the kernels
# stream their arrays once, so the traffic grows with the elements); the memory
# traffic is the same in both modes.  k_elem is the mean of its first-stage and
# last-stage (CFL) launches.
DRAM_PER_ELEM = {"k_force": (847900928 + 373555200) / 2097152,
                 "k_elem": (716255232 + 464538624 + 717109760 + 462138624) / 2 / 2097152}
NCU_PER_ELEM = {"exact": {
    "k_force": {"fp64_ops": 124518424 / 262144, "dram_bytes": DRAM_PER_ELEM["k_force"]},
    "k_elem": {"fp64_ops": (157286400 + 169936928) / 2 / 262144, "dram_bytes": DRAM_PER_ELEM["k_elem"]},
}, "fma": {
    "k_force": {"fp64_ops": 88342528 / 262144, "dram_bytes": DRAM_PER_ELEM["k_force"]},
    "k_elem": {"fp64_ops": (127926272 + 137425432) / 2 / 262144, "dram_bytes": DRAM_PER_ELEM["k_elem"]},
}}


def link_rates(nbytes: int = 1 << 30) -> dict:
    """The host link's copy rate, the roofline of the end-to-end transfers:
    cudaMemcpyAsync of one 1 GiB pinned buffer to and from HBM (best of three,
    CUDA events on a side stream)."""
    import torch
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    out = {}
    with torch.cuda.stream(s):
        for name, dst, src in (("h2d_gbs", dev, host), ("d2h_gbs", host, dev)):
            best = None
            for _ in range(4):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                dst.copy_(src, non_blocking=True)
                e1.record(s)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            out[name] = nbytes / (best * 1e-3) / 1e9
    s.synchronize()
    del host, dev
    out["what"] = "cudaMemcpyAsync of a 1 GiB pinned buffer, best of 4; upload_frac / download_frac: the " \
                  "state transfer's bytes / time against it"
    return out


def measure_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU reference
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        p = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10)
        for line in p.stdout.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_reference_sample(args, n: int, cycles: int, warmup: int, strength: str | None = None,
                         threads: int | None = None) -> dict:
    """The reference's own SGH solver (compiled from its sources against the
    MATAR/Kokkos stand-in, OpenMP on every host core unless `threads` is given)
    on a bounded sample of the workload: the same jittered, permuted Sedov
    problem on an n^3 mesh (with the test strength model on every material when
    `strength` is given)."""
    from oracle import build_ref, orc
    if not orc.reference_available("fierro_ref_fast"):
        build_ref.build_reference()
    if not orc.reference_available("fierro_ref_fast"):
        raise RuntimeError("reference executable unavailable (no reference sources on this machine)")
    prob = workload(n, args.seed, getattr(args, "problem", "sedov"))
    if strength:
        from fierro_gb300 import problems
        problems.with_strength(prob, strength, args.shear_modulus)
    cores = threads or os.cpu_count() or 1
    st = orc.run_reference(prob, cycles=cycles, kind="fierro_ref_fast", threads=cores, warmup=warmup)
    secs = st["calc_seconds"]
    return {"value": prob.mesh.num_elems * cycles / secs, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": "%d^3 jittered permuted %s (%d elements), %d cycles timed by the reference's own "
                      "cycle-loop timer after %d warm-up cycles, OMP_NUM_THREADS=%d" %
                      (n, "Noh" if prob.name.startswith("noh") else "Sedov",
                       prob.mesh.num_elems, cycles, warmup, cores),
            "seconds": secs, "cpu_model": cpu_model()}


# ------------------------------------------------------------------ parity
PARITY_FIELDS = ("coords", "vel", "den", "pres", "sie")
POSITIVE_FIELDS = ("den", "pres", "sie")


def parity_error(got, ref, floor: float = 1e-3) -> float:
    """max |got - ref| / max(|ref|, floor * max|ref|): pointwise relative error,
    values below `floor` of the field's peak compared at that scale."""
    import numpy as np
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(got))) if got.size else 0.0
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor * scale)))


def parity_error_tight(got, ref, key: str) -> float:
    """The tight metric: purely relative for the positive fields (density,
    pressure, energy: a 1e-10 background value is compared at its own scale),
    floor 1e-9 of the peak for positions and velocities."""
    import numpy as np
    if key in POSITIVE_FIELDS:
        got = np.asarray(got, dtype=np.float64)
        ref = np.asarray(ref, dtype=np.float64)
        return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)))
    return parity_error(got, ref, 1e-9)


def parity_leg(args, stream) -> dict:
    """The GPU's state, in both arithmetic modes, against the reference's own
    solver (its sources compiled with -ffp-contract=off, the uncontracted
    arithmetic the reference specifies, OpenMP on every host core) on the same
    jittered, permuted deck at the CPU sample's size, after one RK2 cycle and
    after the bench's K cycles: the largest pointwise error of positions,
    velocities, density, pressure and energy in both metrics, and how many values
    differ at all.  The gates are 1e-12 after one cycle and 1e-9 after K."""
    import numpy as np
    from fierro_gb300 import sgh
    from oracle import build_ref, orc
    if not orc.reference_available("fierro_ref"):
        build_ref.build_reference()
    if not orc.reference_available("fierro_ref"):
        raise RuntimeError("reference executable unavailable (no reference sources on this machine)")
    n, K = args.cpu_n, max(2, args.steps)
    prob = workload(n, args.seed, args.problem)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    refs = {c: orc.run_reference(prob, cycles=c, kind="fierro_ref", threads=cores) for c in (1, K)}
    t_ref = time.perf_counter() - t0
    st = sgh.setup(prob)
    out = {"deck": "%d^3 jittered permuted %s, seed %d (the workload's family at the CPU sample's size)"
                   % (n, "Noh" if args.problem == "noh" else "Sedov", args.seed),
           "reference": "the reference's own SGH solver, sources compiled unmodified with -ffp-contract=off "
                        "(oracle/_ref/fierro_ref)",
           "cycles": [1, K], "gates": {"1": 1e-12, str(K): 1e-9},
           "metrics": {"max_err": "max |gpu - ref| / max(|ref|, 1e-3 max|ref|)",
                       "max_err_tight": "density, pressure, energy: max |gpu - ref| / |ref|; positions, "
                                        "velocities: floor 1e-9 max|ref|"},
           "reference_seconds": t_ref}
    ok = True
    for mode_name, mode in (("exact", sgh.FP_EXACT), ("fma", sgh.FP_FMA)):
        res = {}
        with sgh.SGHSolver(prob, fp_mode=mode, stream=stream.cuda_stream) as s:
            s.set_state(st)
            done = 0
            for c in (1, K):
                s.run(c - done)
                done = c
                g = sgh.compared_fields(s.get_state())
                r = refs[c]
                gate = 1e-12 if c == 1 else 1e-9
                e = {k: parity_error(g[k], r[k]) for k in PARITY_FIELDS}
                et = {k: parity_error_tight(g[k], r[k], k) for k in PARITY_FIELDS}
                res["%d_cycles" % c] = {
                    "max_err": e, "max_err_tight": et,
                    "values_differing": {k: int(np.sum(np.asarray(g[k]) != np.asarray(r[k]))) for k in PARITY_FIELDS},
                    "time_rel_err": abs(s.time()[0] - r["time"]) / abs(r["time"]),
                    "within_gate": bool(max(e.values()) <= gate and max(et.values()) <= gate)}
                ok = ok and res["%d_cycles" % c]["within_gate"]
        out[mode_name] = res
    out["all_within_gates"] = ok
    return out


def reference_arm(args):
    dist, rank, world = dist_init(args)
    if rank != 0:
        return
    try:
        ref = run_reference_sample(args, args.cpu_n, max(1, args.steps), args.warmup)
    except Exception as exc:  # pragma: no cover - depends on the machine
        print(json.dumps({"impl": "reference", "unavailable": str(exc).splitlines()[0]}))
        return
    line = {"impl": "reference", "metric": metric_of(args), "value": ref["value"], "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * ref["seconds"] / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(config_of(args), sample_elements=args.cpu_n ** 3),
            "cpu_baseline": {"value": ref["value"], "unit": UNIT, "cores": ref["cores"], "kind": "reference",
                             "sample": ref["sample"]},
            "e2e": {"value": ref["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------ our arm
def ours(args):
    import numpy as np
    import torch
    dist, rank, world = dist_init(args)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    from fierro_gb300 import sgh

    t0 = time.time()
    prob = workload(args.n, args.seed, args.problem)
    st = sgh.setup(prob)
    stream = torch.cuda.Stream()
    mode = sgh.FP_EXACT if args.fp_mode == "exact" else sgh.FP_FMA
    solver = sgh.SGHSolver(prob, fp_mode=mode, stream=stream.cuda_stream)
    solver.set_state(st)
    t_setup = time.time() - t0
    nn, ne = prob.mesh.num_nodes, prob.mesh.num_elems
    fp64_rate = sgh.measure_fp64_rate()
    energy0 = solver.energy()  # IE + KE of the uploaded state (a full-size invariant)

    solver.run(args.warmup)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = ClockSampler(dev)
    clocks.start()
    torch.cuda.synchronize()
    barrier(dist)
    ran, total_ms, kms = solver.run_timed(args.steps)
    torch.cuda.synchronize()
    barrier(dist)
    ck = clocks.stop()
    if ran != args.steps:
        raise RuntimeError("only %d of %d cycles ran (time_final reached)" % (ran, args.steps))
    energy1 = solver.energy()
    t_max = reduce_max(dist, total_ms)
    value = ne * args.steps * world / (t_max * 1e-3)

    # per-kernel device time over the timed region
    names = solver.launch_names()
    per = {}
    for nm, ms in zip(names, kms):
        per[nm] = per.get(nm, 0.0) + ms
    launches = {nm: names.count(nm) * args.steps for nm in set(names)}
    share = {nm: per[nm] / max(total_ms, 1e-9) for nm in per}
    dom = max(("k_force", "k_node", "k_elem"), key=lambda k: per[k])
    nnz = int(solver_neighbor_count(prob))
    dom_ms = per[dom] / launches[dom]
    ab = alg_bytes(dom, nn, ne, nnz)
    hbm_peak, peak_kind = measure_peaks()
    achieved = ab / (dom_ms * 1e-3) / 1e9
    cycle_bytes = sum(alg_bytes(k, nn, ne, nnz) * names.count(k) for k in ("k_force", "k_node", "k_elem"))
    cycle_ms = total_ms / args.steps
    ncu = NCU_PER_ELEM[args.fp_mode]

    # end to end through the C ABI with host buffers: upload the state, run the
    # same K cycles, download the state (copies inside the timed region)
    e2e = None
    if not args.no_e2e:
        # the output arrays exist and are resident, as the state arrays a caller
        # of sgh_solve passes in (and gets back, in place) are
        host = {k: v.copy() for k, v in st.items()}
        h2d = sum(st[k].nbytes for k in ("node_coords", "node_vel", "node_mass", "elem_den", "elem_pres",
                                         "elem_sspd", "elem_sie", "elem_vol", "elem_mass", "elem_mat_id",
                                         "elem_statev", "elem_div", "elem_stress"))
        d2h = sum(host[k].nbytes for k in host if k != "elem_statev" and k != "elem_mat_id")
        # one untimed solve first (the first GPU access to a host page costs a
        # translation-table walk), then three timed K-cycle solves; the median
        # is reported (the host and its memory are shared with other jobs)
        solver.set_state(st)
        solver.run(1)
        solver.get_state(host)
        trials = []
        for _ in range(3):
            torch.cuda.synchronize()
            barrier(dist)
            te0 = time.perf_counter()
            solver.set_state(st)
            tu = time.perf_counter()
            solver.run(args.steps)
            tr = time.perf_counter()
            solver.get_state(host)
            te1 = time.perf_counter()
            barrier(dist)
            trials.append((reduce_max(dist, te1 - te0), tu - te0, tr - tu, te1 - tr))
        trials.sort()
        med = trials[1]
        link = link_rates()
        e2e = {"value": ne * args.steps * world / med[0], "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "upload_s": med[1], "run_s": med[2], "download_s": med[3],
               "link": dict(link, upload_frac=h2d / med[1] / 1e9 / link["h2d_gbs"],
                            download_frac=d2h / med[3] / 1e9 / link["d2h_gbs"]),
               "trials_s": [[round(x, 4) for x in t] for t in trials],
               "path": "fierro_sgh_set_state + fierro_sgh_run(K) + fierro_sgh_get_state, host buffers in "
                       "the reference layouts (AoS, caller numbering, resident pages), one upload and one "
                       "download per K-cycle solve, the GPU reading and writing the host arrays over "
                       "NVLink-C2C; one untimed warm-up solve, median of three timed solves (trials_s: "
                       "total, upload, run, download); bytes per step = per solve / K"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = run_reference_sample(args, args.cpu_n, args.cpu_cycles, 1)
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": "unavailable: " + str(exc).splitlines()[0]}
        if cpu.get("value") and not args.no_cpu_1thread:
            # the same sample on one host thread (two timed cycles after one warm-up)
            try:
                one = run_reference_sample(args, args.cpu_n, 2, 1, threads=1)
                cpu["one_thread"] = {"value": one["value"], "unit": UNIT, "cores": 1, "sample": one["sample"]}
            except Exception as exc:
                cpu["one_thread"] = {"value": None, "sample": "unavailable: " + str(exc).splitlines()[0]}

    parity = None
    if rank == 0 and world == 1 and not args.no_parity:
        try:
            parity = parity_leg(args, stream)
        except Exception as exc:
            parity = {"unavailable": str(exc).splitlines()[0]}

    if rank != 0:
        return
    line = {
        "metric": metric_of(args), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(config_of(args), fp_mode=args.fp_mode),
        "gpu_launches": int(solver.launches_per_cycle * args.steps),
        "e2e": e2e,
        "roofline": {
            "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak,
            "traffic": ncu[dom]["dram_bytes"] * ne if dom in ncu else None,
            "peak_kind": peak_kind, "alg_bytes_per_launch": ab, "avg_launch_ms": dom_ms,
            "cycle_alg_bytes": cycle_bytes, "cycle_hbm_gbs": cycle_bytes / (cycle_ms * 1e-3) / 1e9,
            "binding_pipe": "fp64",
            "fp64": None if dom not in ncu else {
                "achieved": ncu[dom]["fp64_ops"] * ne / (dom_ms * 1e-3) / 1e9,
                "peak": fp64_rate / 1e9, "unit": "G FP64 thread-instructions/s",
                "frac": ncu[dom]["fp64_ops"] * ne / (dom_ms * 1e-3) / fp64_rate,
                "peak_kind": "measured DFMA rate on this GPU (fierro_measure_fp64_rate)",
                "ops_per_elem": ncu[dom]["fp64_ops"]},
        },
        "kernels": {nm: {"launches": launches[nm], "ms": per[nm], "share": share[nm]} for nm in sorted(per)},
        "cpu_baseline": None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                                     "cpu_model", "one_thread") if k in cpu},
        "parity": parity,
        "invariants": {
            "total_energy_rel_change": abs(sum(energy1) - sum(energy0)) / abs(sum(energy0)),
            "total_energy": [sum(energy0), sum(energy1)], "cycles": args.warmup + args.steps,
            "what": "IE + KE of the full-size state before the warm-up and after the timed cycles (the SGH update "
                    "is compatible: total energy is conserved up to rounding, sgh_solve.cpp:686-688)"},
        "clocks": ck,
        "setup_seconds": t_setup,
        "device_bytes": solver.device_bytes,
    }
    solver.close()
    if args.fp_mode == "fma" and not args.no_exact_leg and world == 1:
        # the same timed cycles in the exact mode (the reference's arithmetic bit
        # for bit), for comparison
        with sgh.SGHSolver(prob, fp_mode=sgh.FP_EXACT, stream=stream.cuda_stream) as sx:
            sx.set_state(st)
            sx.run(args.warmup)
            ran_x, total_x, kms_x = sx.run_timed(args.steps)
            names_x = sx.launch_names()
        per_x = {}
        for nm, ms in zip(names_x, kms_x):
            per_x[nm] = per_x.get(nm, 0.0) + ms
        line["exact_mode"] = {"value": ne * ran_x / (total_x * 1e-3), "ms_per_step": total_x / max(ran_x, 1),
                              "kernels_ms_per_launch": {nm: per_x[nm] / (names_x.count(nm) * max(ran_x, 1))
                                                        for nm in per_x}}
    # the other two measured forms of the path, in the same run: the batched
    # ensemble (512 instances against looping the plain solver) and the discrete
    # adjoint (cost against the plain forward, gradient against differences)
    if world == 1 and not args.no_batch_leg:
        try:
            line["batch"] = batch_measure(args, modes=("fma", "exact"))
        except Exception as exc:
            line["batch"] = {"unavailable": str(exc).splitlines()[0]}
    if world == 1 and not args.no_adjoint_leg:
        try:
            line["adjoint"] = adjoint_measure(args, compact=True)
        except Exception as exc:
            line["adjoint"] = {"unavailable": str(exc).splitlines()[0]}
    print(json.dumps(line))


def solver_neighbor_count(prob) -> int:
    """nnz of the element-neighbour lists of a structured box (elements sharing a
    node): interior 26, fewer on faces, edges and corners."""
    m = prob.mesh
    n = round(m.num_elems ** (1.0 / 3.0))
    if n ** 3 != m.num_elems:
        return 26 * m.num_elems
    per_axis_sum = (n - 2) * 3 + 2 * 2 if n >= 2 else 1  # sum over i of (#neighbours along the axis incl. self)
    return per_axis_sum ** 3 - m.num_elems


def batch_workload(n_inst: int, seed: int, cycles: int):
    """The ensemble: instance i is Sedov or Noh with probability 1/2, a uniform
    n^3 box with n ~ U{8..48}, gamma ~ U[1.2, 1.8]; Sedov deposits E ~ logU[0.05, 5]
    in the origin element, Noh flows in at speed ~ U[0.5, 2].  Seeded through the
    counter-based generator of fierro_gb300.mesh."""
    import math
    from fierro_gb300 import mesh, problems
    out = []
    for i in range(n_inst):
        u = mesh.uniform01(seed, 1000 + i, 5)
        n = 8 + min(40, int(u[1] * 41))
        gamma = 1.2 + 0.6 * float(u[2])
        if u[0] < 0.5:
            energy = math.exp(math.log(0.05) + float(u[3]) * (math.log(5.0) - math.log(0.05)))
            out.append(problems.sedov(n, energy=energy, gamma=gamma, cycles=cycles))
        else:
            speed = 0.5 + 1.5 * float(u[4])
            out.append(problems.noh(n, speed=-speed, gamma=gamma, cycles=cycles))
    return out


def batch_measure(args, modes=None) -> dict:
    """Config 4: the ensemble through fierro_batch_run against looping the plain
    solver over the same instances, in each arithmetic mode of `modes`: the
    default launch shape, the shape fierro_batch_autotune picks, and (first mode)
    the instances reordered smallest first; clocks sampled over the timed runs."""
    import torch
    from fierro_gb300 import sgh
    torch.cuda.set_device(0)
    modes = modes or (args.fp_mode,)
    probs = batch_workload(args.instances, args.seed, args.batch_cycles)
    states = [sgh.setup(p) for p in probs]
    ne_tot = sum(p.mesh.num_elems for p in probs)
    n = len(probs)
    out = {"metric": "batched SGH ensemble instances/s (%d Sedov/Noh instances, n~U{8..48}, %d cycles each)"
                     % (n, args.batch_cycles), "unit": "instances/s", "elements_total": ne_tot,
           "config": {"workload": "ensemble", "instances": n, "cycles": args.batch_cycles, "seed": args.seed,
                      "launches_per_cycle": 8, "timing": "host wall clock around fierro_batch_run / "
                      "fierro_sgh_run (each synchronises); the autotuner's own time is reported apart"}}

    def run_batch(ps, sts, mode, tune):
        stream = torch.cuda.Stream()
        b = sgh.Batch(ps, fp_mode=mode, stream=stream.cuda_stream)
        for i, st in enumerate(sts):
            b.set_state(i, st)
        tuned = None
        if tune:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            chosen, log = b.autotune(cycles=3)
            tuned = {"shape": list(chosen), "autotune_s": time.perf_counter() - t0,
                     "candidates": [[list(sh), ms] for sh, ms in log]}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run(args.batch_cycles)
        dt = time.perf_counter() - t0
        cyc = [b.time(i)[2] for i in range(len(ps))]
        shape = b.shape()
        b.close()
        return dt, cyc, shape, tuned

    clocks = ClockSampler(0)
    clocks.start()
    for k, mname in enumerate(modes):
        mode = sgh.FP_EXACT if mname == "exact" else sgh.FP_FMA
        with sgh.Batch(probs[:2], fp_mode=mode) as w:  # load the batch kernels
            w.set_state(0, states[0])
            w.set_state(1, states[1])
            w.run(3)
        t_batch, cycles_done, shape, _ = run_batch(probs, states, mode, False)
        t_tuned, _, shape_t, tuned = run_batch(probs, states, mode, True)
        # the same instances one after another through the single-problem solver
        t_loop = 0.0
        for p, st in zip(probs, states):
            with sgh.SGHSolver(p, fp_mode=mode) as s1:
                s1.set_state(st)
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                s1.run(args.batch_cycles)
                t_loop += time.perf_counter() - t1
        r = {"value": n / t_batch, "loop_value": n / t_loop, "speedup_vs_loop": t_loop / t_batch,
             "batch_seconds": t_batch, "loop_seconds": t_loop, "shape": list(shape),
             "element_cycles_per_s": sum(p.mesh.num_elems * c for p, c in zip(probs, cycles_done)) / t_batch,
             "instances_stopped_early": int(sum(c < args.batch_cycles for c in cycles_done)),
             "tuned": dict(tuned, value=n / t_tuned, batch_seconds=t_tuned,
                           speedup_vs_loop=t_loop / t_tuned, gain_vs_default=t_batch / t_tuned)}
        if k == 0:
            order = sorted(range(n), key=lambda i: probs[i].mesh.num_elems)
            t_sorted, _, _, _ = run_batch([probs[i] for i in order], [states[i] for i in order], mode, False)
            r["smallest_first"] = {"value": n / t_sorted, "batch_seconds": t_sorted,
                                   "gain_vs_default": t_batch / t_sorted}
        out[mname] = r
    out["clocks"] = clocks.stop()
    return out


def batch_bench(args):
    m = batch_measure(args)
    r = m[args.fp_mode]
    line = {"metric": m["metric"], "value": r["value"], "unit": "instances/s", "higher_is_better": True,
            "dtype": "f64", "data": "synthetic", "loop_value": r["loop_value"],
            "speedup_vs_loop": r["speedup_vs_loop"], "batch_seconds": r["batch_seconds"],
            "loop_seconds": r["loop_seconds"], "elements_total": m["elements_total"],
            "element_cycles_per_s": r["element_cycles_per_s"],
            "instances_stopped_early": r["instances_stopped_early"],
            "config": dict(m["config"], fp_mode=args.fp_mode), "clocks": m["clocks"]}
    print(json.dumps(line))


def adjoint_bench(args):
    print(json.dumps(adjoint_measure(args)))


def adjoint_measure(args, compact: bool = False) -> dict:
    """Discrete adjoint of 400 RK2 cycles of jittered Sedov 64^3: cost of the
    checkpointed forward and of the backward against the plain forward, and the
    gradient against central differences of the GPU forward along seeded
    directions (per-element relative sie perturbations U(-1,1) and a gamma shift
    U(-1,1)), plus the CPU oracle's forward on a 12^3, 100-cycle deck."""
    import numpy as np
    import torch
    from fierro_gb300 import adjoint, problems, sgh
    torch.cuda.set_device(0)
    n, cyc, k = args.adj_n, args.adj_cycles, args.adj_ckpt
    target = adjoint.sedov_target(n, cyc, jitter=0.1, seed=7)
    prob = problems.sedov(n, jitter=0.1, seed=7, cycles=cyc)
    dm = adjoint.DensityMismatch(prob, target, cyc, ckpt_every=k)
    s = dm.solver
    J0, sb, gb, vb = dm.gradient()  # warm-up (allocates the tape)
    s.adj_verify(True)
    dm.gradient()
    vstats = s.adj_stats()
    s.adj_verify(False)
    t_plain, t_fwd, t_bwd = [], [], []
    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(max(args.steps, 1) if args.steps < 5 else 3):
        s.set_state(dm.state0)
        s.synchronize()
        t0 = time.perf_counter()
        s.run(cyc)
        t_plain.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        dm.forward()
        t_fwd.append(time.perf_counter() - t0)
        seed = 2.0 * dm.mass * (dm.last_den - dm.target)
        t0 = time.perf_counter()
        sb2, gb2, _ = s.adj_backward(den=seed)
        t_bwd.append(time.perf_counter() - t0)
    tp, tf, tb = min(t_plain), min(t_fwd), min(t_bwd)
    # the frozen-branch check: central differences (step 1e-6) of the forward
    # with the base run's switch decisions held, along the seeded directions;
    # the three-point difference carries a truncation error h^2 J3 / 6 (J3 the
    # third derivative along the direction), the five-point one (same step, two
    # more forwards) O(h^4)
    Jf, sbf, gbf, _ = dm.gradient_frozen()
    frozen = []
    for d_sie, d_g in dm.directions(args.adj_dirs, seed=args.seed):
        ad = float(np.dot(sbf, d_sie) + np.sum(gbf) * d_g)
        # the directional derivative's own conditioning: the sum of its terms'
        # magnitudes against its value (a direction nearly orthogonal to the
        # gradient has a small derivative and FD rounding noise of the usual size)
        mag = float(np.sum(np.abs(sbf * d_sie)) + abs(np.sum(gbf) * d_g))
        fd3, fd5 = dm.fd5(d_sie, d_g, h=1e-6)
        frozen.append({"ad": ad, "fd3": fd3, "fd5": fd5, "rel3": abs(fd3 - ad) / abs(fd3),
                       "rel5": abs(fd5 - ad) / abs(fd5), "cancellation": mag / abs(ad),
                       "rel5_of_terms": abs(fd5 - ad) / mag})
    dm.unfreeze()
    rel3 = np.array([d["rel3"] for d in frozen]) if frozen else np.zeros(0)
    rel5 = np.array([d["rel5"] for d in frozen]) if frozen else np.zeros(0)

    def summary(rel):
        return {"max_rel": float(rel.max()) if rel.size else None,
                "median_rel": float(np.median(rel)) if rel.size else None,
                "within_1e-6": int((rel <= 1e-6).sum())}

    worst = max(frozen, key=lambda d: d["rel5"]) if frozen else None
    fd_frozen = {"directions": len(frozen), "step": 1e-6, "five_point": summary(rel5),
                 "three_point": summary(rel3),
                 "five_point_max_rel_of_terms": max(d["rel5_of_terms"] for d in frozen) if frozen else None,
                 "worst_direction": None if worst is None else {k: worst[k] for k in ("ad", "fd5", "rel5",
                                                                                    "cancellation")},
                 "gradient_equals_plain": bool(np.array_equal(sbf, sb) and np.array_equal(gbf, gb)),
                 "what": "central differences at step 1e-6 (three-point and five-point stencils) of the "
                         "frozen-branch forward (fierro_adj_branches FREEZE: the limiter neighbour and clamps, Mach "
                         "switch, compression sign and |div| sign, Riemann-velocity guard, CFL element and node "
                         "pair, dt growth cap and clamps held at the base run's decisions)"}
    if not compact:
        fd_frozen["per_direction"] = frozen
    dirs = []
    for d_sie, d_g in ([] if compact else dm.directions(args.adj_dirs, seed=args.seed)):
        ad = float(np.dot(sb, d_sie) + np.sum(gb) * d_g)
        fd6 = dm.fd(d_sie, d_g, h=1e-6)
        est, h, spread, _ = dm.fd_consistent(d_sie, d_g)
        dirs.append({"ad": ad, "fd_h1e-6": fd6, "rel_h1e-6": abs(fd6 - ad) / abs(fd6), "fd": est, "h": h,
                     "fd_spread": spread, "rel": abs(est - ad) / abs(est)})
    fd_check, orc_rel = None, None
    if dirs:
        rel = np.array([d["rel"] for d in dirs])
        spread = np.array([d["fd_spread"] for d in dirs])
        clean = spread <= 1e-6
        fd_check = {"directions": len(dirs), "max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
                    "within_1e-6": int((rel <= 1e-6).sum()),
                    "fd_self_consistent": int(clean.sum()),
                    "max_rel_where_fd_self_consistent": float(rel[clean].max()) if clean.any() else None,
                    "all_within_fd_spread": bool(np.all(rel <= np.maximum(spread, 1e-6))),
                    "h1e-6_max_rel": float(max(d["rel_h1e-6"] for d in dirs)),
                    "per_direction": dirs}
        # the reference algorithm's forward on the CPU (oracle), smaller deck
        dm12 = adjoint.DensityMismatch(problems.sedov(12, jitter=0.1, seed=7, cycles=100),
                                       adjoint.sedov_target(12, 100, jitter=0.1, seed=7), 100, ckpt_every=13)
        J12, sb12, gb12, _ = dm12.gradient()
        orc_rel = []
        try:
            from oracle import orc
            f = orc.density_mismatch_forward(dm12)
            for d_sie, d_g in dm12.directions(3, seed=args.seed):
                ad = float(np.dot(sb12, d_sie) + np.sum(gb12) * d_g)
                fd = dm12.fd(d_sie, d_g, h=1e-6, forward=f)
                orc_rel.append(abs(fd - ad) / abs(fd))
        except Exception as exc:  # oracle not built on this machine
            orc_rel = ["unavailable: %s" % str(exc).splitlines()[0]]
    line = {"metric": "discrete adjoint cost: backward / plain forward (Sedov %d^3, %d RK2 cycles, FP64)" % (n, cyc),
            "value": tb / tp, "unit": "x plain forward", "higher_is_better": False, "dtype": "f64",
            "data": "synthetic", "forward_plus_backward_x": (tf + tb) / tp, "checkpointed_forward_x": tf / tp,
            "plain_forward_s": tp, "adj_forward_s": tf, "backward_s": tb,
            "J": J0, "replay_force_mismatches": vstats["force_mismatches"], "status": vstats["status"],
            "dt_cycles": {"cfl": vstats["dt_cfl_cycles"], "growth": vstats["dt_growth_cycles"],
                          "other": vstats["dt_other_cycles"]},
            "adjoint_device_bytes": vstats["device_bytes"], "tape_bytes": vstats["tape_bytes"],
            "checkpoint_bytes": vstats["ckpt_bytes"],
            "fd_frozen": fd_frozen,
            "fd_check": fd_check,
            "oracle_fd_check_12cubed_100cycles": orc_rel,
            "config": {"workload": "adjoint sedov%d jitter0.1 seed7" % n, "cycles": cyc, "ckpt_every": k,
                       "objective": "sum_e M_e (rho_e - rho_target_e)^2, rho_target from origin energy 0.3",
                       "params": "per-element initial sie and gamma", "fd": "central, steps 1e-5..1e-8; "
                       "the reported step is the one agreeing best with the next smaller step",
                       "timing": "host wall clock around fierro_sgh_run / fierro_adj_forward / "
                       "fierro_adj_backward (each synchronises), best of 3"}}
    line["clocks"] = clocks.stop()
    return line


def outputs_bench(args):
    """Graphics dumps (EnSight Gold + element state text, the reference's formats)
    every 25 cycles of 200 on jittered Sedov 64^3 with a 16-slot snapshot ring:
    wall time of fierro_sgh_run with the writer thread on against off (the cycle
    loop's cost of dumping), the time the writer needed after the last cycle
    (flush), and the writer's text throughput.  The dumps go to a temporary
    directory."""
    import shutil
    import tempfile
    import torch
    from fierro_gb300 import problems, sgh
    torch.cuda.set_device(0)
    n, cyc = 64, 200
    p = problems.sedov(n, jitter=0.1, seed=7, cycles=cyc)
    p.params.graphics_cyc_ival = 25
    st = sgh.setup(p)
    res = {}
    with sgh.SGHSolver(p) as s:
        s.set_state(st)
        s.run(5)
        for mode in ("off", "on", "off"):
            d = tempfile.mkdtemp(prefix="fierro_out_")
            s.set_output(d if mode == "on" else None, slots=16)
            s.set_state(st)
            s.synchronize()
            t0 = time.perf_counter()
            s.run(cyc)
            s.synchronize()
            t1 = time.perf_counter()
            dumps = s.flush_output()
            t2 = time.perf_counter()
            size = sum(os.path.getsize(os.path.join(a, f)) for a, _, fs in os.walk(d) for f in fs)
            res.setdefault(mode, []).append({"run_s": t1 - t0, "flush_s": t2 - t1, "dumps": dumps, "bytes": size})
            s.set_output(None)
            shutil.rmtree(d, ignore_errors=True)
    off = min(r["run_s"] for r in res["off"])
    on = res["on"][0]
    line = {"metric": "cycle-loop wall time with graphics dumps on / off (Sedov 64^3, 200 cycles, dump every 25)",
            "value": on["run_s"] / off, "unit": "x", "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "run_off_s": off, "run_on_s": on["run_s"], "writer_tail_s": on["flush_s"], "dumps": on["dumps"],
            "bytes_written": on["bytes"], "writer_bytes_per_s": on["bytes"] / (on["run_s"] + on["flush_s"]),
            "slots": 16,
            "config": {"workload": "sedov64 jitter0.1 seed7", "cycles": cyc, "graphics_cyc_ival": 25,
                       "formats": "EnSight Gold (case, geo, 9 scalars, 2 vectors) + element state text",
                       "timing": "host wall clock around fierro_sgh_run (synchronised)"}}
    print(json.dumps(line))


# The same per-element counters for the strength instantiations, from an ncu
# capture of the 64^3 case (exact mode, mean of the two RK-stage launches): hypo
# k_force<0,0,1>, hyper k_elem<*,0,1>.
NCU_PER_ELEM_STRENGTH = {
    ("hypo", "k_force"): {"fp64_ops": (195035144 + 200802328) / 2 / 262144,
                          "dram_bytes": (125629952 + 36976128 + 144625152 + 37889536) / 2 / 262144},
    ("hyper", "k_elem"): {"fp64_ops": (206307328 + 218957856) / 2 / 262144,
                          "dram_bytes": (109707008 + 43060480 + 109892864 + 43815680) / 2 / 262144},
}


def strength_alg_bytes(kind: str, kernel: str, nn: int, ne: int, nnz: int) -> float:
    """Compulsory bytes of one launch (mean over the two RK stages) of a kernel of
    a strength run with every element on the model: the plain kernel's bytes plus
    the stress rows (9 doubles per bin), the cycle-start energy and the shear
    modulus column the model reads.  Hypo: the force pass reads stress(1) and
    stress(0) and writes stress(1) on both stages.  Hyper: the force pass reads
    stress(1) and copies it on the first stage; the element pass reads both bins
    and writes stress(1)."""
    base = alg_bytes(kernel, nn, ne, nnz)
    if kind == "hypo" and kernel == "k_force":
        return base + ne * (72 + 72 + 72 + 8 + 8)
    if kind == "hyper" and kernel == "k_force":
        return base + ne * (72 + 36)
    if kind == "hyper" and kernel == "k_elem":
        return base + ne * (72 + 72 + 72 + 8 + 8)
    return base


def strength_bench(args):
    """The strength-model path at scale: the benchmark workload with every
    material on the shipped hypo-elastic model (as a hypo or hyper model), timed
    with per-launch CUDA events like the plain run, against the same problem
    without strength in the same process, plus the reference CPU solver running
    the same model on a bounded sample."""
    import numpy as np
    import torch
    from fierro_gb300 import problems, sgh
    torch.cuda.set_device(0)
    mode = sgh.FP_EXACT if args.fp_mode == "exact" else sgh.FP_FMA
    res = {}
    for kind in ("none", args.strength):
        prob = workload(args.n, args.seed)
        if kind != "none":
            problems.with_strength(prob, kind, args.shear_modulus)
        st = sgh.setup(prob)
        nn, ne = prob.mesh.num_nodes, prob.mesh.num_elems
        with sgh.SGHSolver(prob, fp_mode=mode) as s:
            s.set_state(st)
            s.run(args.warmup)
            clocks = ClockSampler(0)
            clocks.start()
            ran, total_ms, kms = s.run_timed(args.steps)
            ck = clocks.stop()
            if ran != args.steps:
                raise RuntimeError("only %d of %d cycles ran" % (ran, args.steps))
            names = s.launch_names()
            per = {}
            for nm, ms in zip(names, kms):
                per[nm] = per.get(nm, 0.0) + ms
            out = s.get_state() if kind != "none" else None
            res[kind] = {"value": ne * args.steps / (total_ms * 1e-3), "ms_per_step": total_ms / args.steps,
                         "kernels_ms_per_launch": {k: per[k] / (names.count(k) * args.steps) for k in per},
                         "clocks": ck, "device_bytes": s.device_bytes,
                         "launches": int(s.launches_per_cycle * args.steps)}
            if out is not None:
                res[kind]["max_abs_stress"] = float(np.abs(out["elem_stress"][1]).max())
                res[kind]["finite"] = bool(np.isfinite(out["node_coords"]).all())
        nnz = int(solver_neighbor_count(prob))
    r, plain = res[args.strength], res["none"]
    per = r["kernels_ms_per_launch"]
    dom = max(("k_force", "k_node", "k_elem"), key=lambda k: per[k])
    ab = strength_alg_bytes(args.strength, dom, nn, ne, nnz)
    hbm_peak, peak_kind = measure_peaks()
    achieved = ab / (per[dom] * 1e-3) / 1e9
    nc = NCU_PER_ELEM_STRENGTH.get((args.strength, dom)) if args.fp_mode == "exact" else None
    fp64_rate = sgh.measure_fp64_rate()
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = run_reference_sample(args, args.cpu_n, args.cpu_cycles, 1, strength=args.strength)
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": "unavailable: " + str(exc).splitlines()[0]}
    line = {"metric": "SGH element-cycles/s with the %s strength model, %d^3 perturbed Sedov, FP64 RK2"
                      % (args.strength, args.n),
            "value": r["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": dict(config_of(args), fp_mode=args.fp_mode, strength=args.strength,
                           shear_modulus=args.shear_modulus, model="linear hypo-elastic (sgh_user_mat.cuh)"),
            "gpu_launches": r["launches"],
            "plain_value": plain["value"], "strength_over_plain_time": plain["value"] / r["value"],
            "kernels_ms_per_launch": {"strength": per, "plain": plain["kernels_ms_per_launch"]},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": nc["dram_bytes"] * ne if nc else None,
                         "peak_kind": peak_kind, "alg_bytes_per_launch": ab, "avg_launch_ms": per[dom],
                         "binding_pipe": "fp64",
                         "fp64": None if nc is None else {
                             "achieved": nc["fp64_ops"] * ne / (per[dom] * 1e-3) / 1e9, "peak": fp64_rate / 1e9,
                             "unit": "G FP64 thread-instructions/s",
                             "frac": nc["fp64_ops"] * ne / (per[dom] * 1e-3) / fp64_rate,
                             "peak_kind": "measured DFMA rate on this GPU (fierro_measure_fp64_rate)",
                             "ops_per_elem": nc["fp64_ops"]}},
            "max_abs_stress": r["max_abs_stress"], "finite": r["finite"],
            "cpu_baseline": None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind",
                                                                         "sample")},
            "clocks": r["clocks"], "device_bytes": r["device_bytes"]}
    print(json.dumps(line))


def rz_alg_bytes(kind: str, nn: int, ne: int, nnz: int) -> float:
    """Compulsory HBM bytes of one launch of each 2D-RZ kernel (FP64 state, int32
    connectivity, every array touched counted once, gathers at perfect reuse)."""
    if kind == "k_force":
        return ne * (16 + 40 + 4 + 4 + 64) + 4 * nnz + nn * 32
    if kind == "k_node":
        return nn * (4 + 8 + 8 + 1 + 32 + 8 + 32 + 24 + 8) + ne * (16 + 64)
    if kind == "k_elem":
        return ne * (16 + 64 + 8 + 8 + 8 + 16 + 40) + nn * 56
    return 0.0


def rz_bench(args):
    """The 2D-RZ path at scale: RZ Sedov (the deck of the reference's RZ test:
    gamma 5/3, energy 0.49339 in the origin sphere of radius 1.2/64, the test's
    source on its 64 x 64 mesh, four reflecting planes) on an n x n quad mesh of
    [0,1.2]^2 with interior nodes jittered by U(-0.1h, 0.1h) and element and node
    ids permuted from the seed, exact mode, per-launch CUDA events; the reference
    CPU solver with num_dims = 2 on a bounded sample."""
    import torch
    from fierro_gb300 import problems, sgh
    from oracle import build_ref, orc
    torch.cuda.set_device(0)
    mode = sgh.FP_EXACT if args.fp_mode == "exact" else sgh.FP_FMA
    t0 = time.time()
    prob = problems.sedov_rz(args.rz_n, jitter=0.1, seed=args.seed, permute=True, cycles=10 ** 9,
                             source_radius=1.2 / 64)
    st = sgh.setup(prob)
    nn, ne = prob.mesh.num_nodes, prob.mesh.num_elems
    with sgh.SGHSolver(prob, fp_mode=mode) as s:
        s.set_state(st)
        t_setup = time.time() - t0
        s.run(args.warmup)
        clocks = ClockSampler(0)
        clocks.start()
        ran, total_ms, kms = s.run_timed(args.steps)
        ck = clocks.stop()
        if ran != args.steps:
            raise RuntimeError("only %d of %d cycles ran" % (ran, args.steps))
        names = s.launch_names()
        per = {}
        for nm, ms in zip(names, kms):
            per[nm] = per.get(nm, 0.0) + ms
        launches = {nm: names.count(nm) * args.steps for nm in set(names)}
        dev_bytes = s.device_bytes
        launches_total = int(s.launches_per_cycle * args.steps)
        ie, ke = s.energy()
        # end to end through the C ABI with host buffers (staged transfers on this
        # path): upload, the same K cycles, download; warm-up solve, median of three
        host = {k: v.copy() for k, v in st.items()}
        h2d = sum(st[k].nbytes for k in st if k not in ("corner_force",))
        d2h = sum(host[k].nbytes for k in host if k not in ("elem_statev", "elem_mat_id"))
        s.set_state(st)
        s.run(1)
        s.get_state(host)
        trials = []
        for _ in range(3):
            torch.cuda.synchronize()
            te0 = time.perf_counter()
            s.set_state(st)
            tu = time.perf_counter()
            s.run(args.steps)
            tr = time.perf_counter()
            s.get_state(host)
            te1 = time.perf_counter()
            trials.append((te1 - te0, tu - te0, tr - tu, te1 - tr))
        trials.sort()
        med = trials[1]
        e2e = {"value": ne * args.steps / med[0], "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
               "d2h_bytes_per_step": d2h / args.steps, "upload_s": med[1], "run_s": med[2], "download_s": med[3],
               "path": "fierro_sgh_set_state + fierro_sgh_run(K) + fierro_sgh_get_state with host buffers in the "
                       "reference's 2D layouts (the GPU reading and writing the host arrays over NVLink-C2C); "
                       "median of three"}
    nnz = 8 * ne  # a quad's node-sharing neighbours: 8 inside the mesh
    dom = max(("k_force", "k_node", "k_elem"), key=lambda k: per[k])
    dom_ms = per[dom] / launches[dom]
    ab = rz_alg_bytes(dom, nn, ne, nnz)
    hbm_peak, peak_kind = measure_peaks()
    cpu = None
    if not args.no_cpu_baseline:
        try:
            if not orc.reference_available("fierro_ref_fast"):
                build_ref.build_reference()
            sample = problems.sedov_rz(args.rz_cpu_n, jitter=0.1, seed=args.seed, permute=True,
                                       source_radius=1.2 / 64)
            cores = os.cpu_count() or 1
            r = orc.run_reference(sample, cycles=args.cpu_cycles, kind="fierro_ref_fast", threads=cores, warmup=1)
            cpu = {"value": sample.mesh.num_elems * args.cpu_cycles / r["calc_seconds"], "unit": UNIT, "cores": cores,
                   "kind": "reference",
                   "sample": "%d^2 jittered permuted RZ Sedov (%d quads), num_dims 2, %d cycles timed by the "
                             "reference's own cycle-loop timer after 1 warm-up cycle, OMP_NUM_THREADS=%d"
                             % (args.rz_cpu_n, sample.mesh.num_elems, args.cpu_cycles, cores)}
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "reference",
                   "sample": "unavailable: " + str(exc).splitlines()[0]}
    line = {"metric": "SGH element-cycles/s, 2D-RZ Sedov %d^2 quads, FP64 RK2" % args.rz_n,
            "value": ne * args.steps / (total_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sedov_rz_%d^2_jitter0.1_permuted" % args.rz_n, "elements": ne, "nodes": nn,
                       "source_radius": 1.2 / 64,
                       "gamma": 5.0 / 3.0, "energy": 0.49339, "cfl": 0.4, "rk_stages": 2, "seed": args.seed,
                       "fp_mode": args.fp_mode, "num_dims": 2,
                       "l2": "inputs larger than L2 (device state %.1f GB vs 129 MB L2)" % (dev_bytes / 1e9)},
            "gpu_launches": launches_total, "e2e": e2e,
            "kernels": {nm: {"launches": launches[nm], "ms": per[nm], "share": per[nm] / total_ms} for nm in per},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": ab / (dom_ms * 1e-3) / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": ab / (dom_ms * 1e-3) / 1e9 / hbm_peak, "traffic": None,
                         "peak_kind": peak_kind, "alg_bytes_per_launch": ab, "avg_launch_ms": dom_ms},
            "energy": {"ie": ie, "ke": ke},
            "cpu_baseline": cpu, "clocks": ck, "setup_seconds": t_setup, "device_bytes": dev_bytes}
    print(json.dumps(line))


def configs_bench(args):
    """Sedov 12^3 (200 cycles) and Noh 32^3 (500 cycles, stopping at time_final
    after 325) on the shipped-mesh geometry: the run as graph replays
    (fierro_sgh_run, median of three), the same with a CUDA event after every
    launch, the one-shot fierro_sgh_solve with host buffers, and the reference
    CPU solver on all host cores and on one (its own cycle-loop timer)."""
    import torch
    from fierro_gb300 import problems, sgh
    from oracle import build_ref, orc
    torch.cuda.set_device(0)
    if not orc.reference_available("fierro_ref_fast"):
        build_ref.build_reference()
    out = {}
    for name, prob in (("sedov12", problems.sedov(12, geo_digits=5)), ("noh32", problems.noh(32, geo_digits=5))):
        cyc = prob.params.cycle_stop
        ne = prob.mesh.num_elems
        st = sgh.setup(prob)
        with sgh.SGHSolver(prob) as s:
            s.set_state(st)
            s.run(3)
            s.set_state(st)
            ran, total_ms, _ = s.run_timed(cyc)
            # the same run as graph replays (what fierro_sgh_run does), timed around
            # the synchronised call; per-launch events above cost host time per launch
            reps = []
            for _ in range(3):
                s.set_state(st)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.run(cyc)
                reps.append(time.perf_counter() - t0)
            graph_s = sorted(reps)[1]
        host = {k: v.copy() for k, v in st.items()}
        sgh.sgh_solve(prob, host)  # warm-up of the one-shot path
        host = {k: v.copy() for k, v in st.items()}
        t0 = time.perf_counter()
        r = sgh.sgh_solve(prob, host)
        one_shot = time.perf_counter() - t0
        cores = os.cpu_count() or 1
        ref_all = orc.run_reference(prob, kind="fierro_ref_fast", threads=cores)
        ref_one = orc.run_reference(prob, kind="fierro_ref_fast", threads=1)
        # the reference stops at time_final too; both runs take the same cycles
        out[name] = {"elements": ne, "cycles": ran,
                     "gpu_graph_element_cycles_per_s": ne * ran / graph_s, "gpu_graph_s": graph_s,
                     "gpu_events_element_cycles_per_s": ne * ran / (total_ms * 1e-3), "gpu_events_ms": total_ms,
                     "gpu_one_shot_element_cycles_per_s": ne * r["cycles"] / one_shot, "gpu_one_shot_s": one_shot,
                     "cpu_element_cycles_per_s": ne * ran / ref_all["calc_seconds"], "cpu_cores": cores,
                     "cpu_1core_element_cycles_per_s": ne * ran / ref_one["calc_seconds"],
                     "time_final_gpu": r["time_value"], "time_final_cpu": ref_all["time"]}
    print(json.dumps({"metric": "small reference decks: element-cycles/s, GPU and reference CPU", "unit": UNIT,
                      "dtype": "f64", "data": "synthetic (generator equal to the shipped meshes)",
                      "configs": out}))


def fp64_peak_bench(args):
    """FP64 operations per second of a pure stream against chains per thread,
    threads per block and blocks per SM, fma / add / mul."""
    import torch
    from fierro_gb300 import sgh
    torch.cuda.set_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    rows = []
    for threads, bps in ((128, 1), (128, 2), (128, 4), (128, 8), (256, 1), (256, 4), (256, 8), (512, 4), (1024, 2)):
        row = {"threads": threads, "blocks_per_sm": bps}
        for ch in (1, 2, 4, 8, 16):
            row["fma_ch%d" % ch] = sgh.fp64_stream_rate(ch, 0, threads, bps) / 1e9
        row["add_ch8"] = sgh.fp64_stream_rate(8, 1, threads, bps) / 1e9
        row["mul_ch8"] = sgh.fp64_stream_rate(8, 2, threads, bps) / 1e9
        rows.append(row)
    peak = max(max(v for k, v in r.items() if k not in ("threads", "blocks_per_sm")) for r in rows)
    print(json.dumps({"metric": "FP64 pipe throughput, pure stream", "unit": "G FP64 thread-instructions/s",
                      "value": peak, "higher_is_better": True, "dtype": "f64", "rows": rows,
                      "clocks": clocks.stop()}))


def main(argv=None):
    args = parse(argv)
    if args.fp64_peak:
        fp64_peak_bench(args)
        return
    if args.configs:
        configs_bench(args)
        return
    if args.rz:
        rz_bench(args)
        return
    if args.strength:
        strength_bench(args)
        return
    if args.outputs:
        outputs_bench(args)
        return
    if args.adjoint:
        adjoint_bench(args)
        return
    if args.batch:
        batch_bench(args)
        return
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
