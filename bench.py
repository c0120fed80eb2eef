"""Benchmark: stiffness (K) assembly throughput on the 3D Hooke workload
"unit cube, structured 40x40x40 hex27, 3x3x3 Gauss, E=2.1e5, nu=0.3"
(1,594,323 DoFs, 297,685,449 structural CSC entries), in GNNZ/s = structural
nnz / assembly time with the CSC pattern prebuilt.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|fp32q]
  python bench.py --impl reference ...   CPU restatement of the reference's
                                          threaded direct-CSC assembly

One JSON line on stdout (rank 0).  Fields follow the repository's bench
contract: value (device-resident inputs, CUDA events on the launching
stream), e2e (through the C-ABI from pinned host buffers: mesh upload +
assembly + CSC copy-back), roofline of the dominant kernel, cpu_baseline,
clocks sampled during the timed region, gpu_launches.

The timed steps repeat the assembly of the same operator on the same mesh:
the mesh's affine geometry and the pattern's stored layout come from the
warm-up (every value and row index is computed again, and every column's
count is checked against the layout).  without_layout_reuse times the same
steps with LLF_STORED_LAYOUT=0; other_form, general_geometry (the mesh
turned off its axes), precision_form_error and samples (batched, serving,
the config-2 end-to-end solve) are reported beside the headline.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 40
ORDER = 2
E, NU = 2.1e5, 0.3
WORKLOAD = "hooke3d-unit-cube-hex27-40x40x40"


def workload_name(n):
    """The workload label for n cells per edge (the headline case is 40)."""
    return f"hooke3d-unit-cube-hex27-{n}x{n}x{n}"
# ncu DRAM bytes (read + write) of one FP64 assembly of hex27 16^3 (19,320,201
# structural nnz): k_affine_geometry 1.3 MB, k_elem_affine 153.8 MB (the
# general-geometry k_elem_fp64 165.0 MB), k_colgather 338.2 MB, k_compact 417.5 MB
NNZ_16CUBE = 19320201
KERNEL_DRAM_BYTES_16CUBE = {"k_affine_geometry": 1.324032e6, "k_elem_fp64": (6.096128 + 158.8992) * 1e6,
                            "k_elem_affine": (0.392704 + 153.449984) * 1e6,
                            "k_colgather": (224.209664 + 114.00704) * 1e6, "k_compact": (165.33248 + 252.210688) * 1e6,
                            # the gather compacting into the pattern's kept stored layout (both launches)
                            "k_colgather_layout": (179.443968 + 174.397696 + 58.287104 + 7.202048) * 1e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "fp32q"])
    ap.add_argument("--n", type=int, default=N_CELLS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="assembly", choices=["assembly", "batched", "serving", "tl"])
    ap.add_argument("--instances", type=int, default=512, help="batched: instances (the first k of the seeded 512)")
    ap.add_argument("--batched-form", default="fp64", choices=["fp64", "fp32q"],
                    help="batched: assembly form (fp32q misses the 1e-8 displacement target on these systems)")
    ap.add_argument("--batched-solve", default="fp64", choices=["fp64", "mixed"],
                    help="batched: CG precision (mixed: FP32 iterations, 1.1-1.7x the FP64 products here)")
    ap.add_argument("--batched-reltol", type=float, default=1e-10, help="batched: CG relative residual")
    ap.add_argument("--group-nnz", type=float, default=1.0e9,
                    help="batched: structural entries of one group")
    ap.add_argument("--streams", type=int, default=3, help="batched: groups in flight (one CUDA stream each)")
    ap.add_argument("--requests", type=int, default=200, help="serving: requests of the Poisson stream")
    ap.add_argument("--workers", type=int, default=8,
                    help="serving: preparation threads (engine) or solver workers (pool)")
    ap.add_argument("--server", default="engine", choices=["engine", "pool"],
                    help="serving: continuous-batching engine or the worker pool")
    ap.add_argument("--max-systems", type=int, default=256, help="serving: engine slots")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: offered requests per second (Poisson)")
    ap.add_argument("--one-sample", type=int, default=0,
                    help="serving: the one-at-a-time arm on the first k requests (0: all)")
    ap.add_argument("--no-peak", action="store_true", help="skip the DGEMM FP64 reference rate")
    ap.add_argument("--no-other-form", action="store_true", help="skip the second arithmetic form")
    ap.add_argument("--no-tune", action="store_true", help="assembly: skip the schedule autotuner")
    ap.add_argument("--no-c4b", action="store_true", help="tl: skip the hex125 12^3 Newton solve")
    ap.add_argument("--c4b-fp64", action="store_true", help="tl: also run the hex125 Newton with the FP64 tangent")
    ap.add_argument("--no-samples", action="store_true",
                    help="assembly line: skip the short batched and serving samples")
    ap.add_argument("--no-plain", action="store_true", help="batched: skip the one-at-a-time plain arm")
    ap.add_argument("--profile", action="store_true", help="batched: add a traced pass's kernel time breakdown")
    ap.add_argument("--precond", default=None, choices=["jacobi", "bjacobi", "ic0", "auto"],
                    help="CG preconditioner (defaults: ic0 for batched, bjacobi for tl, auto for serving: "
                         "Jacobi for its scalar heat requests)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device="cuda") -> float:
    """The largest x over the job's ranks (the job's step time is its
    slowest rank's); x itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, units: float, ms_step: float) -> float:
    """Whole-job rate in units / ns (GNNZ/s for structural entries): every
    rank assembles its own replica of the workload ("replicas only", weak
    scaling), so the job moves world * units per step of the slowest rank."""
    return world * units / (ms_step * 1e-3) / 1e9


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.tmp:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(rows), "reasons": sorted(reasons)}


# ----------------------------------------------------------------- workload
def algorithmic(mesh, nnz, aligned=True):
    """Algorithmic bytes of one assembly (structural nnz values written, node
    coordinates and connectivity read) and FP64 operations of the element
    kernel under the arithmetic contract (FMA = 2 flops).  Every element of
    the structured mesh passes the affinity test, so the count is the affine
    form's: affinity test, Jacobian inverse and per-element coefficients,
    then per node pair Ksym = W S (ns x ns FMA), Kanti = U A (na x na FMA,
    a != b) and the 2 na additions that form the two off-diagonal halves.
    Its elements are axis-aligned bricks (aligned=True): W is then zero
    outside its d x d diagonal-component block and its mixed diagonal, U is
    diagonal, and the kernel performs d x d FMA plus 2 na products per pair
    (the coefficients: 2 ns + 3 d + d (d - 1) + 2 na + d + 1 operations)."""
    npe, d = mesh.npe, 3
    ns, na = (6, 3) if d == 3 else (3, 1)
    bytes_ = 8 * nnz + 24 * mesh.non + 4 * npe * mesh.nel
    npairs = npe * (npe + 1) // 2
    test = 2 * d * d * npe + npe * d * (1 + 3 * d)
    inverse = 42
    if aligned:
        coeffs = 2 * ns + 3 * d + d * (d - 1) + 2 * na + d + 1
        pairs = (npairs - npe) * (2 * d * d + 2 * na + 2 * na) + npe * (2 * d * d + na)
    else:
        coeffs = 3 * ns * ns + (2 + 1) * ns * ns + d * ns * 2 + 5 * na * na + ns + 1
        pairs = (npairs - npe) * (2 * ns * ns + 2 * na * na + 2 * na) + npe * 2 * ns * ns
    flops = mesh.nel * (test + inverse + coeffs + pairs)
    return bytes_, flops


L2_NOTE = "GPU arm: a 256 MB buffer (> 129 MB L2) written before every timed step"


def structural_nnz_hex27(n, nz=None):
    """Structural CSC entries of the n x n x nz hex27 box for 3 DoFs per node:
    along one axis of 2n+1 lattice nodes a vertex shares cells with 5
    nodes (3 on the boundary) and a mid node with 3, and two nodes share an
    element iff they share a cell along every axis, so the node-pair count is
    a product of the per-axis counts."""
    nz = n if nz is None else nz
    c1 = lambda m: 2 * 3 + (m - 1) * 5 + m * 3
    return 9 * c1(n) * c1(n) * c1(nz)


def workload_config(n, form="fp64"):
    """The config object both arms print (identical keys and values)."""
    return {"workload": workload_name(n), "elements": n ** 3, "dofs": 3 * (2 * n + 1) ** 3,
            "structural_nnz": structural_nnz_hex27(n), "form": form, "l2": L2_NOTE}


class CpuBaseline:
    """The reference's element arithmetic on the host cores: per-point
    B^T D B (src/linear.jl:190-330) with the threaded direct-CSC scatter of
    its DSL assembly (src/multifield.jl:2394-2499), restated in C with
    OpenMP (oracle/llfem_oracle.c, orc_assemble_bdb_threaded), on a slab
    n x n x k of the same mesh (the workload and tables from oracle/, not
    from the GPU library).  The slab is sized from a first (warm) run so that
    one run takes about run_s."""

    def __init__(self, orc, run_s=4.0, n=N_CELLS):
        from oracle import workload as wk
        self.orc, self.wk, self.n = orc, wk, n
        self.threads = orc.num_threads()
        self.rule = wk.hex27_rule()
        self._slab(2)
        t = self.run()
        self._slab(int(max(1, min(n, round(2 * run_s / max(t, 1e-3))))))
        self.run()   # warm at size

    def _slab(self, k):
        self.k = k
        self.xyz, self.conn = self.wk.box_hex27(self.n, k / self.n)
        self.pat = self.orc.pattern(self.xyz.shape[0], self.conn, 3)

    def run(self):
        return self.orc.assemble_bdb_threaded(0, 3, self.xyz, self.conn, self.rule, E, NU, self.pat,
                                              nthreads=self.threads)

    def report(self, ts):
        t = statistics.median(ts)
        ta = statistics.median([self.orc.assemble_threaded(self.orc.ELASTIC, 0, 3, 3, self.xyz, self.conn, self.rule,
                                                           [E, NU], self.pat, nthreads=self.threads)
                                for _ in range(2)])
        nnz, n, k = self.pat.nnz, self.n, self.k
        return {"value": nnz / t / 1e9, "unit": "GNNZ/s", "cores": self.threads, "kind": "port",
                "sample": f"{n}x{n}x{k} hex27 slab of the same mesh ({self.conn.shape[0]} elements, {nnz} structural "
                          f"nnz), median of {len(ts)} warm runs of {t:.2f} s: the reference's per-point B'DB element "
                          f"arithmetic (src/linear.jl:190-330) with its threaded direct-CSC scatter "
                          f"(src/multifield.jl:2394-2499), restated in C/OpenMP",
                "affine_restatement": {"value": nnz / ta / 1e9, "unit": "GNNZ/s", "seconds": ta,
                                       "what": "the oracle's node-pair affine form (the GPU's arithmetic contract, "
                                               "2.39 GFLOP at 40^3 against ~136 GFLOP of B'DB), same slab"}}


def cpu_baseline(orc, runs=3):
    b = CpuBaseline(orc)
    ts = [b.run() for _ in range(runs)]
    return b.report(ts), statistics.median(ts)


def run_reference(args):
    """The CPU reference arm: loads only the oracle (oracle/_build), never
    the GPU library.  A step is one run of the bounded slab sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    from oracle import oracle as orc
    orc.build()
    b = CpuBaseline(orc, run_s=2.5)
    for _ in range(args.warmup):
        b.run()
    secs = [b.run() for _ in range(args.steps)]
    info = b.report(secs)
    v = info["value"]
    out = {"metric": "K-assembly throughput (structural nnz / s)", "value": v, "unit": "GNNZ/s",
           "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": statistics.median(secs) * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic structured mesh (unit cube)", "config": workload_config(args.n),
           "cpu_baseline": info, "e2e": {"value": v, "unit": "GNNZ/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def _pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(math.ceil(q / 100.0 * len(v))) - 1)] if v else None


NNZ_PER_DOF_TET10 = 83   # structural entries per DoF of the tet10 boxes (the 16-instance sample: 82.8)


def batched_groups(inst, budget_nnz):
    """Instances grouped so that each group's structural entries (estimated
    from its DoFs) stay within budget_nnz: the batch is admitted to HBM a
    group at a time (about 60 device bytes per entry: values, the stored
    CSC, the IC(0) factor).  Instances are taken by size, so a group holds
    instances of similar size, which need similar CG iteration counts: a
    group's CG runs until its slowest system converges, and systems that
    converged early only idle through the tail."""
    groups, cur, acc = [], [], 0
    order = sorted(range(len(inst)), key=lambda k: inst[k][0].non)
    for k in order:
        m = inst[k][0]
        est = NNZ_PER_DOF_TET10 * 3 * m.non
        if cur and acc + est > budget_nnz:
            groups.append(cur)
            cur, acc = [], 0
        cur.append(k)
        acc += est
    if cur:
        groups.append(cur)
    return groups


def run_batched(args, llf):
    """Batched configuration: independent tet10 boxes (element counts
    log-uniform 1e3-2e5, seeded), admitted to the GPU in groups by their
    footprint; per group one assembly launch (FP32 quadrature, FP64
    accumulation by default) and one segmented mixed-precision PCG (FP32
    iterations, FP64 reliable updates, IC(0); CUDA graph) to an FP64
    relative residual.  Solves/s over all instances, the relative
    displacement error of sample instances against a direct solve of the
    FP64-assembled matrix, and the plain GPU form (each instance alone, FP64
    assembly + FP64 Jacobi-PCG) on the same instances."""
    import numpy as np
    import torch
    from llfem_gb300 import workloads as wl
    rng = np.random.default_rng(wl.SEED)
    inst = [wl.batched_instance(rng) for _ in range(args.instances)]
    prec = args.precond or "ic0"
    form = args.batched_form
    mixed = args.batched_solve == "mixed"
    reltol = args.batched_reltol
    groups = batched_groups(inst, args.group_nnz)
    built = []
    for g in groups:
        batch, noff = llf.concat_meshes([inst[k][0] for k in g])
        mats = [llf.Material(f"body#{i}", E=inst[k][1], nu=inst[k][2]) for i, k in enumerate(g)]
        # each group on a context (CUDA stream) of its own, so that groups on
        # different streams overlap (one group's assembly and factorisation
        # with another's CG)
        P = llf.Problem(mats, type="Solid", mesh=batch, device=0 if args.streams > 1 else None)
        f = llf.loadVector(P, [llf.load(f"right#{i}", fx=1.0) for i in range(len(g))])
        sup = [llf.displacementConstraint(f"left#{i}", ux=0, uy=0, uz=0) for i in range(len(g))]
        P.pattern()
        built.append((g, P, f, sup, noff))

    def run_group(item):
        g, P, f, sup, noff = item
        K = llf.stiffnessMatrix(P, precision=form)
        u = llf.solveFieldBatched(K, f, support=sup, node_offsets=noff, preconditioner=prec, reltol=reltol,
                                  precision="mixed" if mixed else "fp64")
        del K
        return (u, None)

    def one_pass(keep=False):
        if args.streams <= 1:
            return [run_group(item) for item in built]
        # args.streams groups in flight, each on its own stream (threads: the
        # library calls release the interpreter)
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=args.streams) as ex:
            return list(ex.map(run_group, built))

    times = []
    res = None
    for rep in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = one_pass()
        torch.cuda.synchronize()
        if rep >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    kernels_ms = None
    if args.profile:
        # one more pass with the library's per-launch event tracing (graph
        # replay off while tracing): the kernel time breakdown of a pass
        ctx = built[0][1]._ctx
        ctx.profile_reset()
        ctx.profile(True)
        one_pass()
        torch.cuda.synchronize()
        ctx.profile(False)
        kernels_ms = {k: round(v["ms"], 3) for k, v in sorted(ctx.profile_report().items(), key=lambda kv: -kv[1]["ms"])}
    its = np.concatenate([u.iterations for u, _ in res])
    # accuracy against the FP64-assembled matrix of each checked instance (the
    # plain form's matrix, bit-identical to the oracle's): a direct solve for
    # the smallest instance of every group (up to 30k DoFs: sparse LU of 3D
    # elasticity fills in fast), an FP64 PCG to 1e-14 for the largest one
    import scipy.sparse.linalg as spla
    errs = []
    sizes = [inst[k][0].non for k in range(len(inst))]
    check = sorted({min(g, key=lambda k: sizes[k]) for g in groups})[:4]
    for k in check + [int(np.argmax(sizes))]:
        gi = next(ix for ix, (g, *_rest) in enumerate(built) if k in g)
        g, P, f, sup, noff = built[gi]
        i = g.index(k)
        a, b = 3 * noff[i], 3 * noff[i + 1]
        m, E, nu = inst[k]
        llf.set_current(m)
        Pi = llf.Problem([llf.Material("body", E=E, nu=nu)], type="Solid", mesh=m)
        fi = f.a[a:b, 0]
        fixed = np.zeros(b - a, bool)
        fixed[llf.constrainedDoFs(Pi, [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]) - 1] = True
        fr = ~fixed
        ud = np.zeros(b - a)
        if b - a <= 30000:
            how = "direct (scipy spsolve)"
            Ki = llf.stiffnessMatrix(Pi).A
            ud[fr] = spla.spsolve(Ki.tocsc()[fr][:, fr].tocsc(), fi[fr])
        else:
            how = "FP64 PCG (IC(0)) to 1e-14"
            Kd = llf.stiffnessMatrix(Pi)
            ud = llf.solveFieldBatched(Kd, fi, support=[llf.displacementConstraint("left", ux=0, uy=0, uz=0)],
                                       preconditioner="ic0", reltol=1e-14, maxiter=40 * (b - a)).a[:, 0]
            del Kd
        errs.append({"instance": int(k), "dofs": int(b - a), "against": how,
                     "rel_err": float(np.linalg.norm(res[gi][0].a[a:b, 0] - ud) / np.linalg.norm(ud))})
    # the plain GPU form: every instance on its own, FP64 assembly and
    # Jacobi-PCG (FP64) to the same tolerance, one after the other (patterns
    # built before the timed loop, as for the batch)
    plain = None
    if not args.no_plain:
        singles = []
        for i, (m, E, nu) in enumerate(inst):
            llf.set_current(m)
            Pi = llf.Problem([llf.Material("body", E=E, nu=nu)], type="Solid", mesh=m)
            Pi.pattern()
            singles.append((Pi, llf.loadVector(Pi, [llf.load("right", fx=1.0)]),
                            [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]))

        def solve_one(Pi, fi, si):
            Ki = llf.stiffnessMatrix(Pi)
            return llf.solveField(Ki, fi, support=si, iterative=True, preconditioner="jacobi", reltol=reltol,
                                  maxiter=20 * 3 * Pi.non)
        solve_one(*singles[int(np.argmin([m.nel for m, _, _ in inst]))])   # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for Pi, fi, si in singles:
            solve_one(Pi, fi, si)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        plain = {"value": len(inst) / tp, "unit": "solves/s", "seconds": tp,
                 "form": f"one instance at a time: FP64 assembly + FP64 Jacobi-PCG to {reltol:g}",
                 "speedup_of_batched": (len(inst) / t) / (len(inst) / tp)}
    nel = sum(m.nel for m, _, _ in inst)
    return {"metric": "batched assemble+solve (independent tet10 systems / s)", "value": len(inst) / t,
            "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("f32-quadrature/f64-accumulate" if form == "fp32q" else "f64") + " assembly, "
                     + ("f32 iterations/f64 reliable updates" if mixed else "f64") + " CG",
            "data": f"synthetic: seeded tet10 boxes ({len(inst)} of the 512-instance workload)",
            "config": {"workload": f"batched-tet10-{len(inst)}", "instances": len(inst), "elements": nel,
                       "dofs": int(3 * sum(sizes)), "groups": len(groups), "group_nnz_budget": args.group_nnz,
                       "groups_in_flight": args.streams,
                       "structural_nnz": int(sum(P.pattern().nnz for _, P, *_ in built)), "precond": prec,
                       "reltol": reltol, "assembly": form, "solve": args.batched_solve},
            "cg_iterations": {"min": int(its.min()), "median": float(np.median(its)), "max": int(its.max())},
            "rel_err_vs_direct": errs, "max_rel_err_vs_direct": max(e["rel_err"] for e in errs),
            "plain_gpu": plain, "kernels_ms_traced_pass": kernels_ms}


def run_c2_solve(llf, n, reltol=1e-10):
    """Config 2 end to end through the public API (the reference's
    stiffnessMatrix, massMatrix, loadVector and solveDisplacement,
    src/linear.jl:70-87, :1843-2004, :3088-3434, :3711-3870): hex27 n^3 unit
    cube, E = 2.1e5, nu = 0.3, rho = 7.85e-9; K and the consistent M in FP64;
    face x = 0 clamped, face x = 1 under a uniform traction of 1 along x;
    IC(0)-preconditioned CG to a relative residual of reltol.  The solution's
    true residual on the free DoFs is measured with the library's product,
    and M's entries must sum to 3 rho V (V = 1)."""
    import numpy as np
    llf.structured_box_mesh(n=n, order=ORDER)
    mat = llf.Material("body", E=E, nu=NU, rho=7.85e-9)
    P = llf.Problem([mat], type="Solid")
    P.device_mesh()
    P.pattern()
    ctx = P._ctx
    ts = {}
    t0 = time.perf_counter()
    K = llf.stiffnessMatrix(P)
    ctx.sync()
    ts["stiffness_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    M = llf.massMatrix(P, lumped=False)
    ctx.sync()
    ts["mass_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    f = llf.loadVector(P, [llf.load("right", fx=1.0)])
    ts["load_s"] = time.perf_counter() - t0
    sup = [llf.displacementConstraint("left", ux=0, uy=0, uz=0)]
    t0 = time.perf_counter()
    u = llf.solveDisplacement(K, f, support=sup, iterative=True, reltol=reltol, preconditioner="ic0",
                              maxiter=20 * P.non)
    ts["solve_s"] = time.perf_counter() - t0
    fixed = np.zeros(3 * P.non, dtype=bool)
    fixed[llf.constrainedDoFs(P, sup) - 1] = True
    fa = f.a[:, 0]
    r = (fa - K.dm.spmv(u.a[:, 0]))[~fixed]
    msum = float(M.dm.copy_csc()[2].sum())
    return {"workload": workload_name(n) + "-clamped-traction", "dofs": 3 * P.non, "stored_nnz_K": K.nnz(),
            "stored_nnz_M": M.nnz(), "precond": "ic0", "reltol": reltol, "cg_iterations": int(u.iterations),
            "relres_reported": float(u.relres),
            "true_relres_free": float(np.linalg.norm(r) / np.linalg.norm(fa[~fixed])),
            "mass_sum_rel_err": abs(msum - 3 * 7.85e-9) / (3 * 7.85e-9),
            **ts, "total_s": sum(ts.values())}


def run_serving(args, llf):
    """Serving configuration: a Poisson stream (200 req/s) of steady heat
    requests through llf_server; p50/p99 latency and solves/s, against the same
    requests solved one at a time."""
    import numpy as np
    import threading
    from llfem_gb300 import workloads as wl
    rng = np.random.default_rng(wl.SEED)
    meshes = {}
    reqs = [wl.heat_request(rng, cache=meshes) for _ in range(args.requests)]
    arrivals = np.cumsum(rng.exponential(1.0, size=len(reqs))) / args.rate

    def precond(m):
        mode = args.precond or "auto"
        if mode == "auto":
            # Jacobi for these scalar (one unknown per node) requests: IC(0)
            # saves only ~1.7x the iterations of a Laplacian, and a scalar
            # sweep has one FMA per list position, so its colour launches are
            # mostly latency (the whole stream: 22.7 solves/s with IC(0) from
            # 50k nodes, 40.4 with Jacobi).  IC(0) pays on vector problems
            # (the batched elasticity: 3x fewer iterations, 1.6x faster).
            return llf._lib.PRECOND_JACOBI
        return {"jacobi": llf._lib.PRECOND_JACOBI, "bjacobi": llf._lib.PRECOND_BJACOBI,
                "ic0": llf._lib.PRECOND_IC0}[mode]

    def submit(srv, r):
        m, k, fixed, x0 = r
        return srv.submit_heat(m.dim, m.xyz, m.conn, m.family, m.order, k, x0, fixed, reltol=1e-10,
                               precond=precond(m))

    # one at a time (a single worker, next request after the previous result)
    warm = [wl.heat_request(np.random.default_rng(1), dofs_max=5e3) for _ in range(2 * args.workers)]
    one = llf._lib.Server(workers=1)
    one.wait(submit(one, warm[0]))
    n_one = len(reqs) if args.one_sample <= 0 else min(len(reqs), args.one_sample)
    t0 = time.perf_counter()
    for r in reqs[:n_one]:
        one.wait(submit(one, r))
    t_single = time.perf_counter() - t0
    one.close()
    srv = llf._lib.Server(workers=args.workers, budget_bytes=120 << 30, batched=args.server == "engine",
                          max_systems=args.max_systems)
    for t in [submit(srv, r) for r in warm]:   # every worker has created its context
        srv.wait(t)
    tickets = [None] * len(reqs)
    start = time.perf_counter()

    def producer():
        for i, r in enumerate(reqs):
            delay = start + arrivals[i] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            tickets[i] = (submit(srv, r), time.perf_counter())

    th = threading.Thread(target=producer)
    th.start()
    lat, iters = [], []
    done_at = start
    for i in range(len(reqs)):
        while tickets[i] is None:
            time.sleep(0.0005)
        x, it, rr, l, svc = srv.wait(tickets[i][0])
        lat.append(l)
        iters.append(it)
        done_at = max(done_at, time.perf_counter())
    th.join()
    stats = srv.stats()
    timing = srv.timing()
    srv.close()
    span = done_at - start
    dofs = [m.non for m, _, _, _ in reqs]
    return {"metric": f"served steady-heat solves / s (Poisson {args.rate:g} req/s)", "value": len(reqs) / span,
            "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": 1, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic heat requests (seeded)",
            "config": {"workload": f"serving-heat-{len(reqs)}", "requests": len(reqs), "workers": args.workers,
                       "server": args.server, "max_systems": args.max_systems,
                       "dofs_median": float(np.median(dofs)), "dofs_max": int(max(dofs)), "reltol": 1e-10,
                       "precond": args.precond or "auto"},
            "latency_s": {"p50": _pct(lat, 50), "p99": _pct(lat, 99), "max": max(lat)},
            "offered_req_per_s": args.rate, "stream_s": float(arrivals[-1]),
            "one_at_a_time_solves_per_s": n_one / t_single, "one_at_a_time_sample": n_one,
            "cg_iterations_median": float(np.median(iters)), "peak_device_bytes": stats["peak_bytes"],
            "server_timing": timing}


def run_tl(args, llf):
    """Hyperelastic Total Lagrangian configuration: compressible neo-Hookean
    (mu=1, lambda=10) unit cube hex8 48^3, 30% axial stretch in 10 load steps,
    full Newton with the consistent tangent reassembled every iteration; and
    the tangent assembly of the order-4 hex variant (12^3 hex125)."""
    import numpy as np
    import torch
    prm = {"mu": 1.0, "lambda": 10.0}
    n = 48 if args.n == N_CELLS else args.n
    m = llf.structured_box_mesh(n=n, order=1)
    P = llf.Problem([llf.Material("body")], type="Solid")
    sup = [llf.displacementConstraint("left", ux=0.0), llf.displacementConstraint("right", ux=0.3),
           llf.displacementConstraint("bottom", uy=0.0), llf.displacementConstraint("rear", uz=0.0)]
    P.pattern()
    ctx = P._ctx
    ctx.profile_reset()
    ctx.profile(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = llf.solveDeformation(P, support=sup, params=prm, steps=10, tol=1e-8, preconditioner=args.precond or "bjacobi")
    torch.cuda.synchronize()
    t_newton = time.perf_counter() - t0
    ctx.profile(False)
    prof = ctx.profile_report()
    its = len(u.history)
    # order-4 hex tangent assembly
    m4 = llf.structured_box_mesh(n=12, order=4)
    P4 = llf.Problem([llf.Material("body")], type="Solid")
    F4 = llf.grad(llf.VectorField(np.zeros((3 * m4.non, 1)), P4), add_identity=True)
    P4.pattern()
    llf.tangentMatrix(P4, F4, params=prm)
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        llf.tangentMatrix(P4, F4, params=prm)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t1)
    t4 = min(ts)
    flops4 = 2 * 375 ** 2 * 6 * 125 * m4.nel / 2  # upper-triangle pairs of B^T (D B) per point
    # the same tangent on the tensor cores (tcgen05, split TF32): per element one
    # GEMM 375 x 375 x (15 rows x 125 points), three split products
    ktc = llf.tangentMatrix(P4, F4, params=prm, precision="tf32x3")
    torch.cuda.synchronize()
    ctx.profile(True)
    ctx.profile_reset()
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        ktc = llf.tangentMatrix(P4, F4, params=prm, precision="tf32x3")
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t1)
    ctx.profile(False)
    prof_tc = {k: v["ms"] / max(v["launches"], 1) for k, v in ctx.profile_report().items()}
    t4tc = min(ts)
    k64 = llf.tangentMatrix(P4, F4, params=prm).dm.copy_structural()
    dtc = float(np.abs(ktc.dm.copy_structural() - k64).max() / np.abs(k64).max())
    gemm4 = 2 * 375 ** 2 * (15 * 125) * m4.nel
    tc_ms = prof_tc.get("k_tl_tangent_tc", 0.0)
    # the order-4 variant's Newton solve: hex125 12^3, 30% stretch in 10
    # steps, FP64 residuals, the tangent on the tensor cores (and optionally
    # the FP64 tangent for comparison)
    newton4 = {}
    forms4 = [] if args.no_c4b else (["tf32x3", "fp64"] if args.c4b_fp64 else ["tf32x3"])
    for tform in forms4:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        u4 = llf.solveDeformation(P4, support=sup, params=prm, steps=10, tol=1e-8,
                                  preconditioner=args.precond or "bjacobi", tangent=tform)
        torch.cuda.synchronize()
        tn4 = time.perf_counter() - t1
        last = {}
        for h in u4.history:
            last[h["step"]] = h
        newton4[tform] = {"s": tn4, "newton_iterations": len(u4.history),
                          "cg_iterations": int(sum(h.get("cg_iterations", 0) for h in u4.history)),
                          "steps_converged": int(sum("cg_iterations" not in h for h in last.values())),
                          "final_residual": u4.history[-1]["residual"],
                          "u_norm": float(np.linalg.norm(u4.a))}
    if len(newton4) == 2:
        newton4["u_rel_diff_tf32x3_vs_fp64"] = abs(newton4["tf32x3"]["u_norm"] - newton4["fp64"]["u_norm"]) / \
            newton4["fp64"]["u_norm"]
    return {"metric": "TL Newton iteration time (hex8 48^3, 30% stretch, 10 steps)", "value": t_newton / max(its, 1) * 1e3,
            "unit": "ms/iteration", "n_gpus": 1, "steps": its, "warmup": 0, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic unit cube",
            "config": {"workload": "tl-neohooke-hex8-48", "elements": m.nel, "dofs": 3 * m.non,
                       "precond": args.precond or "bjacobi",
                       "newton_iterations": its, "load_steps": 10},
            "newton_total_s": t_newton,
            "kernels_ms": {k: v["ms"] for k, v in prof.items()},
            "final_residual": u.history[-1]["residual"],
            "hex125_tangent": {"elements": m4.nel, "ms": t4 * 1e3, "gflops_fp64": flops4 / t4 / 1e9,
                               "structural_nnz": P4.pattern().nnz,
                               "tensor_core_form": {"ms": t4tc * 1e3, "kernels_ms": prof_tc,
                                                    "gemm_flops": gemm4,
                                                    "tensor_tflops_per_split": gemm4 / (tc_ms * 1e-3) / 1e12 if tc_ms else None,
                                                    "tensor_tflops_issued": 3 * gemm4 / (tc_ms * 1e-3) / 1e12 if tc_ms else None,
                                                    "max_rel_diff_vs_fp64": dtc}},
            "hex125_newton": newton4}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "assembly":
        import torch
        torch.cuda.set_device(0)
        import __graft_entry__ as entry
        llf = entry.load_package()
        fn = {"batched": run_batched, "serving": run_serving, "tl": run_tl}[args.workload]
        print(json.dumps(fn(args, llf)), flush=True)
        return
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    os.environ["LLF_DEVICE"] = str(local)
    import __graft_entry__ as entry
    llf = entry.load_package()
    L = llf._lib
    form = L.FP32Q if args.form == "fp32q" else L.FP64

    mesh = llf.structured_box_mesh(n=args.n, order=ORDER)
    ctx = L.default_context()
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    dm = L.DeviceMesh(ctx, 3, mesh.xyz, mesh.conn, mesh.family, mesh.order)
    t0 = time.perf_counter()
    pat = L.DevicePattern(dm, 3)
    pattern_s = time.perf_counter() - t0
    nnz = pat.nnz
    Ea, nua = L.f64([E]), L.f64([NU])

    # the assembly's launch schedule, tuned on this mesh before the timed
    # region (llf_autotune_stiffness; no choice changes a result bit)
    tuned = {}
    if not args.no_tune:
        for fm_name, fm in (("fp64", L.FP64), ("fp32q", L.FP32Q)):
            if args.no_other_form and fm != form:
                continue
            t_tune = time.perf_counter()
            buf = L.C.create_string_buffer(1 << 16)
            need = L.C.c_int64(0)
            ctx.check(L.lib().llf_autotune_stiffness(ctx.h, dm.h, pat.h, L.SOLID, L.ptr(Ea, L.C.c_double),
                                                      L.ptr(nua, L.C.c_double), 1, 1.0, fm, 2, buf, 1 << 16,
                                                      L.C.byref(need)))
            rep = json.loads(buf.value.decode())
            tuned[fm_name] = {"chosen": rep["chosen"], "ms": rep["ms"], "candidates": len(rep["trials"]),
                              "default_ms": rep["trials"][0]["ms"], "tuning_s": time.perf_counter() - t_tune}

    def assemble(fm=form):
        h = L.C.c_void_p()
        ctx.check(L.lib().llf_assemble_stiffness(ctx.h, dm.h, pat.h, L.SOLID, L.ptr(Ea, L.C.c_double),
                                                 L.ptr(nua, L.C.c_double), 1, 1.0, fm, L.C.byref(h)))
        return L.DeviceMatrix(ctx, h, pat)

    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def measure(fm, steps, warmup):
        """Timed assemblies of form fm: CUDA events on the library's stream,
        L2 flushed before every step, per-kernel event tracing on."""
        for _ in range(warmup):
            Km = assemble(fm)
            del Km
        ctx.sync()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ctx.profile_reset()
        ctx.profile(True)
        evs = []
        stored = 0
        with ClockSampler(local) as clk:
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                Km = assemble(fm)
                with torch.cuda.stream(stream):
                    b.record(stream)
                stored = Km.nnz()
                del Km
                evs.append((a, b))
            torch.cuda.synchronize()
            ctx.sync()
        ctx.profile(False)
        prof = ctx.profile_report()
        launches = ctx.launches()
        ms = [a.elapsed_time(b) for a, b in evs]
        ms_step = max_over_ranks(sum(ms) / len(ms))
        measure.last_steps_ms = ms   # the individual steps of this call
        return ms_step, prof, launches, stored, clk.summary()

    ms_step, prof, launches, stored, clocks = measure(form, args.steps, args.warmup)
    value = job_rate(world, nnz, ms_step)

    bytes_alg, flops = algorithmic(mesh, nnz)
    hbm_peak, peak_kind = peaks()
    # dominant kernel by summed device time in the timed region
    kname, kstat = max(prof.items(), key=lambda kv: kv[1]["ms"])
    # per assembly: a kernel may launch more than once in one assembly (the
    # gather runs one launch per column-degree class)
    k_ms = kstat["ms"] / args.steps
    k_launches = kstat["launches"] / args.steps
    per_kernel = {k: {"launches": v["launches"], "ms_per_launch": v["ms"] / max(v["launches"], 1),
                      "share": v["ms"] / sum(x["ms"] for x in prof.values())} for k, v in prof.items()}
    asm_ms = sum(v["ms"] for v in prof.values()) / args.steps
    achieved = bytes_alg / (asm_ms * 1e-3) / 1e9

    # FP64 rate of the dominant element kernel vs a measured DGEMM
    fp64_peak = None
    try:
        if args.no_peak:
            raise RuntimeError("skipped")
        x = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
        torch.matmul(x, x)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(3):
            s0 = torch.cuda.Event(enable_timing=True); s1 = torch.cuda.Event(enable_timing=True)
            s0.record(); torch.matmul(x, x); s1.record(); torch.cuda.synchronize()
            best = min(best, s0.elapsed_time(s1))
        fp64_peak = 2 * 8192 ** 3 / (best * 1e-3) / 1e12
        del x
    except Exception:
        pass
    ek = prof.get("k_elem_affine") or prof.get("k_elem_fp64") or {}
    elem_ms = ek.get("ms", 0.0) / max(ek.get("launches", 1), 1)
    fp64_achieved = flops / (elem_ms * 1e-3) / 1e12 if elem_ms > 0 else None

    # DRAM traffic of one FP64 assembly from ncu captures of its kernels on
    # hex27 16^3 (profiles/k_*_hex27_16cube.md), scaled by structural nnz
    traffic = traffic_k = None
    if form == L.FP64 and ORDER == 2:
        elem_k = "k_elem_affine" if "k_elem_affine" in prof else "k_elem_fp64"
        layout = "k_compact" not in prof   # every timed assembly wrote into the kept stored layout
        parts = [elem_k, "k_colgather_layout"] if layout else [elem_k, "k_colgather", "k_compact"]
        if "k_affine_geometry" in prof:    # (kept on the mesh after the first assembly)
            parts.insert(0, "k_affine_geometry")
        if all(k in KERNEL_DRAM_BYTES_16CUBE for k in parts):
            traffic = sum(KERNEL_DRAM_BYTES_16CUBE[k] for k in parts) * nnz / NNZ_16CUBE
        kkey = "k_colgather_layout" if (layout and kname == "k_colgather") else kname
        if kkey in KERNEL_DRAM_BYTES_16CUBE:
            traffic_k = KERNEL_DRAM_BYTES_16CUBE[kkey] * nnz / NNZ_16CUBE
    # the contract's figure: the assembly's algorithmic bytes over the
    # dominant kernel's average launch; the whole assembly's figure beside it
    achieved_k = bytes_alg / (k_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": achieved_k, "peak": hbm_peak, "unit": "GB/s", "frac": achieved_k / hbm_peak,
                "peak_source": peak_kind, "traffic": traffic_k,
                "traffic_source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum of {kname} on hex27 16^3 "
                                  f"(profiles/{kkey}*_hex27_16cube.md), "
                                  f"scaled by structural nnz" if traffic_k else None,
                "algorithmic_bytes": bytes_alg, "dominant_kernel": kname, "dominant_ms": k_ms,
                "dominant_launches_per_assembly": k_launches,
                "note": ("the element kernel is bound by the FP64 pipe, not HBM: see fp64" if kname.startswith("k_elem")
                         else "achieved = the assembly's algorithmic bytes over this kernel's time per assembly "
                              "(all its launches); the element kernel's FP64 rate is under fp64"),
                "assembly": {"kernels": "all kernels of one llf_assemble_stiffness", "ms": asm_ms,
                             "achieved": achieved, "frac": achieved / hbm_peak, "traffic": traffic,
                             "traffic_source": "ncu dram bytes of " + ", ".join(parts) + " on hex27 16^3 "
                                               "(profiles/*_hex27_16cube.md), scaled by structural nnz"
                                               if traffic else None},
                "per_kernel": per_kernel,
                "fp64": {"element_kernel_flops": flops, "achieved_tflops": fp64_achieved,
                         "dgemm_peak_tflops_measured": fp64_peak,
                         "frac": (fp64_achieved / fp64_peak) if (fp64_achieved and fp64_peak) else None}}

    # e2e through the C-ABI from pinned host buffers
    e2e = None
    if not args.no_e2e and rank == 0:
        xyz_h = torch.from_numpy(L.f64(mesh.xyz)).pin_memory()
        conn_h = torch.from_numpy(L.i64a(mesh.conn)).pin_memory()
        Km = assemble()
        nnz_s = Km.nnz()
        del Km
        # capacity = structural nnz, as a caller sizes them before the call
        colptr_h = torch.empty(3 * mesh.non + 1, dtype=torch.int64).pin_memory()
        rowval_h = torch.empty(pat.nnz, dtype=torch.int64).pin_memory()
        nzval_h = torch.empty(pat.nnz, dtype=torch.float64).pin_memory()
        P = lambda t, ct: L.C.cast(t.data_ptr(), L.C.POINTER(ct))
        e2e_steps = max(2, min(args.steps, 3))
        got = L.C.c_int64(0)

        def to_host_fused():
            # one call: assembly with each column slab copied out behind the next
            ctx.check(L.lib().llf_assemble_stiffness_csc(
                ctx.h, dm.h, pat.h, L.SOLID, L.ptr(Ea, L.C.c_double), L.ptr(nua, L.C.c_double), 1, 1.0, form,
                pat.nnz, P(colptr_h, L.C.c_int64), P(rowval_h, L.C.c_int64), P(nzval_h, L.C.c_double),
                L.C.byref(got)))

        def to_host_two_calls():
            Km = assemble()
            ctx.check(L.lib().llf_matrix_copy_csc(ctx.h, Km.h, P(colptr_h, L.C.c_int64),
                                                  P(rowval_h, L.C.c_int64), P(nzval_h, L.C.c_double)))
            del Km

        def time_e2e(fn):
            ts = []
            for i in range(1 + e2e_steps):
                ctx.sync()
                t0 = time.perf_counter()
                ctx.check(L.lib().llf_mesh_update(ctx.h, dm.h, P(xyz_h, L.C.c_double), P(conn_h, L.C.c_int64)))
                fn()
                t1 = time.perf_counter()
                if i > 0:
                    ts.append(t1 - t0)
            return statistics.median(ts)

        te = time_e2e(to_host_fused)
        assert got.value == nnz_s
        te2 = time_e2e(to_host_two_calls)
        full = {"value": nnz / te / 1e9, "unit": "GNNZ/s", "ms_per_step": te * 1e3,
                "h2d_bytes_per_step": xyz_h.numel() * 8 + conn_h.numel() * 8,
                "d2h_bytes_per_step": colptr_h.numel() * 8 + 2 * nnz_s * 8,
                "call": "llf_mesh_update + llf_assemble_stiffness_csc (pinned host arrays)",
                "two_call_ms_per_step": te2 * 1e3,
                "two_call": "llf_mesh_update + llf_assemble_stiffness + llf_matrix_copy_csc"}
        # values against the pattern the caller holds: colptr, nzval and one
        # keep bit per structural entry come back; the caller's rowval (the
        # structural rowval filtered by the bits, llf_rowval_from_keep) is
        # rebuilt inside the timed region whenever the bits differ from the
        # previous call's, and the bits are compared every call
        import numpy as np
        _, srow = pat.copy()
        nw = (pat.nnz + 31) // 32
        keep_h = torch.empty(nw, dtype=torch.int32).pin_memory()
        rows_h = torch.empty(pat.nnz, dtype=torch.int64).pin_memory()
        rebuilt = [0]

        changed = L.C.c_int(1)

        def to_host_values():
            ctx.check(L.lib().llf_assemble_stiffness_values(
                ctx.h, dm.h, pat.h, L.SOLID, L.ptr(Ea, L.C.c_double), L.ptr(nua, L.C.c_double), 1, 1.0, form,
                pat.nnz, P(colptr_h, L.C.c_int64), P(nzval_h, L.C.c_double), P(keep_h, L.C.c_uint32),
                L.C.byref(got), L.C.byref(changed)))
            if changed.value:   # the library compared the bits with its previous call's on the device
                n_rows = L.lib().llf_rowval_from_keep(pat.nnz, L.ptr(srow, L.C.c_int64), P(keep_h, L.C.c_uint32),
                                                      P(rows_h, L.C.c_int64))
                assert n_rows == got.value
                rebuilt[0] += 1

        tv = time_e2e(to_host_values)
        assert got.value == nnz_s
        assert torch.equal(rows_h[:nnz_s], rowval_h[:nnz_s])   # the caller's rowval is the stored one
        e2e = {"value": nnz / tv / 1e9, "unit": "GNNZ/s", "ms_per_step": tv * 1e3,
               "h2d_bytes_per_step": xyz_h.numel() * 8 + conn_h.numel() * 8,
               "d2h_bytes_per_step": colptr_h.numel() * 8 + nnz_s * 8 + nw * 4,
               "call": "llf_mesh_update + llf_assemble_stiffness_values (pinned host arrays; the keep bits are "
                       "compared with the previous call's on the device) + llf_rowval_from_keep when they change",
               "rowval_rebuilds": rebuilt[0],
               "full_csc": full}

    # the other arithmetic form on the same workload (reported beside the headline)
    other = None
    if not args.no_other_form:
        ofm = L.FP64 if form == L.FP32Q else L.FP32Q
        oms, oprof, _, ostored, _ = measure(ofm, args.steps, args.warmup)
        other = {"form": "fp64" if ofm == L.FP64 else "fp32q", "value": world * nnz / (oms * 1e-3) / 1e9,
                 "unit": "GNNZ/s", "ms_per_step": oms, "stored_nnz": ostored,
                 "roofline_frac": bytes_alg / (sum(v["ms"] for v in oprof.values()) / args.steps * 1e-3) / 1e9 / hbm_peak,
                 "per_kernel_ms": {k: v["ms"] / max(v["launches"], 1) for k, v in oprof.items()}}

    # the same assembly with stored-layout reuse off: every step counts the
    # non-zeros, scans and compacts, as the first assembly on a pattern does
    first = None
    if not args.no_other_form and rank == 0:
        os.environ["LLF_STORED_LAYOUT"] = "0"
        try:
            fms, fprof, _, fstored, _ = measure(form, args.steps, args.warmup)
        finally:
            del os.environ["LLF_STORED_LAYOUT"]
        first = {"what": "the headline assembly without the stored layout of the previous assembly on the pattern "
                         "(count, scan and compaction every step, as on a pattern's first assembly)",
                 "value": world * nnz / (fms * 1e-3) / 1e9, "unit": "GNNZ/s", "ms_per_step": fms,
                 "stored_nnz": fstored,
                 "per_kernel_ms": {k: v["ms"] / max(v["launches"], 1) for k, v in fprof.items()}}

    # the FP64 form on the same mesh turned about a skew axis through its
    # centre: every element stays affine but none is axis-aligned, so the
    # element kernel runs the full 51-operation node-pair form instead of the
    # 21-operation form of axis-aligned bricks
    general = None
    if not args.no_other_form and rank == 0:
        import numpy as np
        ax = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
        th = 0.3
        Kx = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        Rm = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * (Kx @ Kx)
        dm.update((mesh.xyz - 0.5) @ Rm.T + 0.5, mesh.conn)
        # (two more warm-up steps: the first one finds the aligned mesh's layout
        # and builds its own)
        gms, gprof, _, gstored, _ = measure(L.FP64, args.steps, args.warmup + 2)
        gsteps = list(measure.last_steps_ms)
        dm.update(mesh.xyz, mesh.conn)
        general = {"geometry": "the same mesh turned by 0.3 rad about the axis (1, 2, 3) through its centre "
                               "(affine elements, none axis-aligned)",
                   "form": "fp64", "value": world * nnz / (gms * 1e-3) / 1e9, "unit": "GNNZ/s", "ms_per_step": gms,
                   "steps_ms": gsteps,
                   "value_from_median_step": world * nnz / (statistics.median(gsteps) * 1e-3) / 1e9,
                   "stored_nnz": gstored,
                   "per_kernel_ms": {k: v["ms"] / max(v["launches"], 1) for k, v in gprof.items()}}

    # the precision form against the FP64 values of the same workload: the
    # largest deviation (relative to the largest entry) and the entries it
    # stores fewer (FP64 rounding residue of mathematically zero entries,
    # which cancel to exact zero in FP32 and are then dropped)
    precision = None
    if not args.no_other_form and rank == 0:
        import numpy as np
        K64 = assemble(L.FP64)
        a, n64 = K64.copy_structural(), K64.nnz()
        del K64
        K32 = assemble(L.FP32Q)
        b, n32 = K32.copy_structural(), K32.nnz()
        del K32
        scale = float(np.abs(a).max())
        d = np.abs(b - a)
        dropped = (b == 0) & (a != 0)
        precision = {"form": "fp32q (FP32 quadrature, FP64 accumulation)", "vs": "fp64 form (bit-identical to the oracle)",
                     "max_abs_err_rel_to_max_entry": float(d.max()) / scale,
                     "rel_frobenius_err": float(np.linalg.norm(d) / np.linalg.norm(a)),
                     "stored_nnz_fp64": int(n64), "stored_nnz_fp32q": int(n32),
                     "stored_nnz_difference": int(n64 - n32),
                     "dropped_entries_max_fp64_value_rel_to_max_entry":
                         float(np.abs(a[dropped]).max()) / scale if dropped.any() else 0.0}
        del a, b, d, dropped

    samples = None
    if not args.no_samples and rank == 0 and world == 1:
        import argparse as _ap
        samples = {}
        try:
            bargs = _ap.Namespace(**{**vars(args), "instances": 16, "steps": 1, "warmup": 1, "no_plain": False,
                                     "precond": None, "batched_form": "fp64", "batched_solve": "fp64",
                                     "batched_reltol": 1e-10, "group_nnz": 1.0e9, "streams": 3})
            r = run_batched(bargs, llf)
            samples["batched"] = {k: r[k] for k in ("value", "unit", "ms_per_step", "dtype", "config", "cg_iterations",
                                                    "rel_err_vs_direct", "max_rel_err_vs_direct", "plain_gpu")
                                  if k in r}
        except Exception as ex:
            samples["batched"] = {"error": str(ex)}
        try:
            samples["c2_solve"] = run_c2_solve(llf, args.n)
        except Exception as ex:
            samples["c2_solve"] = {"error": str(ex)}
        try:
            sargs = _ap.Namespace(**{**vars(args), "requests": 100, "precond": None, "server": "engine",
                                     "max_systems": 256, "rate": 200.0, "one_sample": 0})
            r = run_serving(sargs, llf)
            samples["serving"] = {k: r[k] for k in ("metric", "value", "unit", "config", "latency_s",
                                                    "one_at_a_time_solves_per_s", "cg_iterations_median",
                                                    "offered_req_per_s") if k in r}
        except Exception as ex:
            samples["serving"] = {"error": str(ex)}

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            from oracle import oracle as orc
            orc.build()
            cpu, _ = cpu_baseline(orc)
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "error": str(ex)}

    if rank == 0:
        out = {"metric": "K-assembly throughput (structural nnz / s)", "value": value, "unit": "GNNZ/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64" if form == L.FP64 else "f32-quadrature/f64-accumulate",
               "data": "synthetic structured mesh (unit cube)",
               "config": workload_config(args.n, args.form),
               "stored_nnz": stored, "pattern_build_s": pattern_s, "autotune": tuned,
               "parallelism": "replicas" if world > 1 else "single",
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
               "clocks": clocks, "other_form": other, "without_layout_reuse": first, "general_geometry": general,
               "precision_form_error": precision, "samples": samples}
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
