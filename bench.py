#!/usr/bin/env python3
"""FP64 tile-QR throughput on GB300 -- the plain FP64 form of the tile QR.

Workload (one "step"): flat-tree tile QR (geqrt on the diagonal tiles, tsqrt
down each panel, unmqr/tsmqr trailing updates) of one 8192 x 8192 Float64
matrix, tile nb = 256, inner block ib = 32, entries i.i.d. N(0, 1) from a
fixed seed.  metric = algorithmic flops 4/3 n^3 per step / time, in TFLOP/s.

Contract: `python bench.py --gpus N --steps K --warmup W [--impl reference]`
prints ONE JSON line on rank 0.  Multi-GPU runs are replicas (one matrix per
GPU; the single-matrix tile QR is not sharded), so scaling is weak.

Timing: W untimed steps, then K steps between a barrier and a device sync on
both sides, timed with CUDA events on the launching stream, max over ranks.
Each step first restores A from a pristine copy (a 512 MiB device copy that
is inside the timed region); A is larger than L2, so every step streams it.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "nextla.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "tile-QR TFLOP/s (FP64, 8192^2)"
UNIT = "TFLOP/s"
NB, IB = 256, 32
SEED = 20241203


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="tileqr", choices=["tileqr", "reference"])
    p.add_argument("--n", type=int, default=8192, help="matrix order (default: the 8192^2 workload)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--kernel", default=None,
                   choices=["tsmqr", "tsmqr_tc", "tsmqr_wy", "tsqrt", "geqrt", "tile", "tile_f64p", "hqr",
                            "hqr_square", "batched", "larft", "trsm"],
                   help="time one tile kernel alone (for profiling) instead of the workload")
    p.add_argument("--dtype", default="f64", choices=["f64", "f32", "c64", "c128"],
                   help="element type for --kernel and --adjoint-only --adjoint-kernels")
    p.add_argument("--grp", type=int, default=4, help="with --kernel hqr_square: tiles per flat group")
    p.add_argument("--dag-quantum", type=float, default=None,
                   help="with --kernel tile: bucket width of the persistent kernel's priority sort")
    p.add_argument("--no-ls", action="store_true", help="skip the least-squares comparison")
    p.add_argument("--ls-only", action="store_true", help="run only the least-squares comparison")
    p.add_argument("--ls-m", type=int, default=32768)
    p.add_argument("--ls-n", type=int, default=4096)
    p.add_argument("--ls-no-orth", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the batched uneven QR + solve")
    p.add_argument("--batched-only", action="store_true", help="run only the batched uneven QR + solve")
    p.add_argument("--batched-n", type=int, default=4096, help="problems per batch")
    p.add_argument("--batched-no-tune", action="store_true",
                   help="default (ib, strip) per size class instead of the autotuner's choice")
    p.add_argument("--no-adjoint", action="store_true", help="skip the differentiable QR")
    p.add_argument("--adjoint-only", action="store_true", help="run only the differentiable QR")
    p.add_argument("--adjoint-kernels", action="store_true",
                   help="with --adjoint-only: the forward and adjoint kernels alone, seeded cotangents")
    p.add_argument("--adjoint-shape", default="256,2048,256",
                   help="with --adjoint-only --adjoint-kernels: batch,m,n (a smaller case for profiling)")
    p.add_argument("--no-tall", action="store_true", help="skip the tall-skinny flat vs tree comparison")
    p.add_argument("--tall-only", action="store_true", help="run only the tall-skinny flat vs tree comparison")
    p.add_argument("--no-complex", action="store_true", help="skip the complex tile QR")
    p.add_argument("--no-extras", action="store_true", help="skip the 1024^2 latency and the tiling sweep")
    p.add_argument("--latency-only", action="store_true", help="run only the 1024^2 latency line")
    p.add_argument("--complex-only", action="store_true", help="run only the complex tile QR")
    p.add_argument("--complex-n", type=int, default=4096, help="order of the complex matrix")
    return p.parse_args()


def kernel_bench(args):
    """One tile kernel alone at the tile driver's shapes: tsmqr on a row band
    (256 x (n - 256) pair of tiles rows), tsqrt / geqrt on one 256 x 256 tile."""
    import torch

    import tileqr as tq
    import tileqr_build
    tileqr_build.build()
    tq.set_blocking(False)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    n = args.n
    res = {}
    if args.dag_quantum is not None:
        from tileqr import _lib
        _lib.lib().tqr_tile_dag_order_quantum(args.dag_quantum)
    if args.kernel in ("tile", "tile_f64p"):
        # the persistent tile QR of an n x n matrix in the chosen precision
        # (FP32: its tsmqr updates on the tensor cores; tile_f64p: FP32 with
        # the mixed solve's FP64 panels; complex: 4 real flops per complex one)
        dt = {"f32": torch.float32, "f64": torch.float64, "c64": torch.complex64,
              "c128": torch.complex128}[args.dtype]
        if args.kernel == "tile_f64p":
            dt = torch.float32
        A0 = tq.empty(n, n, dtype=dt)
        if dt.is_complex:
            A0.copy_(torch.complex(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"),
                                   torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")))
        else:
            A0.copy_(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
        A = tq.empty(n, n, dtype=dt)

        def run():
            A.copy_(A0)
            if args.kernel == "tile_f64p":
                tq.tile_geqrf_f64p(A, NB, IB)
            else:
                tq.tile_geqrf(A, NB, IB)
        fl = flops_square(n) * (4 if dt.is_complex else 1)
    elif args.kernel == "hqr":
        # the hierarchical tall-skinny QR (groups of HQR_GRP tiles) of an
        # n x 512 matrix, one persistent launch over its task graph
        dt = torch.float32 if args.dtype == "f32" else torch.float64
        A0 = tq.empty(n, 512, dtype=dt)
        A0.copy_(torch.randn(n, 512, generator=g, dtype=torch.float64, device="cuda"))
        A = tq.empty(n, 512, dtype=dt)

        def run():
            A.copy_(A0)
            tq.tile_geqrf_tree(A, NB, IB, dag=True, grp=HQR_GRP)
        fl = 2.0 * n * 512 ** 2 - 2.0 * 512 ** 3 / 3
    elif args.kernel == "hqr_square":
        # the n x n tile QR on the hierarchical tree (groups of --grp tiles,
        # the leaders by the binary tree), one persistent launch (complex:
        # 4 real flops per complex one)
        dt = {"f32": torch.float32, "f64": torch.float64, "c64": torch.complex64,
              "c128": torch.complex128}[args.dtype]
        A0 = tq.empty(n, n, dtype=dt)
        if dt.is_complex:
            A0.copy_(torch.complex(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"),
                                   torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")))
        else:
            A0.copy_(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
        A = tq.empty(n, n, dtype=dt)

        def run():
            A.copy_(A0)
            tq.tile_geqrf_tree(A, NB, IB, dag=True, grp=args.grp)
        fl = flops_square(n) * (4 if dt.is_complex else 1)
    elif args.kernel == "batched":
        # one launch of the batched uneven QR + solve over --batched-n seeded
        # problems (m ~ U[32,512], n ~ U[16,m], k ~ U[1,8]) in the chosen type
        from tileqr import batched as Bt
        dt = {"f32": torch.float32, "f64": torch.float64, "c64": torch.complex64,
              "c128": torch.complex128}[args.dtype]
        ms, ns, ks = Bt.random_sizes(args.batched_n, seed=SEED)
        bg = Bt.BatchedGels(ms, ns, ks, dtype=dt, tune=not dt.is_complex)
        if dt.is_complex:
            A0 = torch.complex(torch.randn(bg.A.shape, generator=g, dtype=torch.float64, device="cuda"),
                               torch.randn(bg.A.shape, generator=g, dtype=torch.float64, device="cuda")).to(dt)
            B0 = torch.complex(torch.randn(bg.B.shape, generator=g, dtype=torch.float64, device="cuda"),
                               torch.randn(bg.B.shape, generator=g, dtype=torch.float64, device="cuda")).to(dt)
        else:
            A0 = torch.randn(bg.A.shape, generator=g, dtype=torch.float64, device="cuda").to(dt)
            B0 = torch.randn(bg.B.shape, generator=g, dtype=torch.float64, device="cuda").to(dt)

        def run():
            bg.A.copy_(A0)
            bg.B.copy_(B0)
            bg.run(sync=False)
        fl = bg.flops() * (4 if dt.is_complex else 1)
    elif args.kernel == "larft":
        # stand-alone larft!('F', 'C') on an n x 32 block of reflectors
        dt = torch.float32 if args.dtype == "f32" else torch.float64
        V = tq.empty(n, IB, dtype=dt)
        V.copy_(torch.randn(n, IB, generator=g, dtype=torch.float64, device="cuda") / 16)
        tau = torch.rand(IB, generator=g, dtype=torch.float64, device="cuda").to(dt) + 1
        T = tq.zeros(IB, IB, dtype=dt)
        run = lambda: tq.larft("F", "C", n, IB, V, tau, T)
        fl = 1.0 * n * IB * IB
    elif args.kernel == "trsm":
        # the least-squares back-solve R X = B, n x n upper R, 4 right-hand sides
        R = tq.empty(n, n)
        R.copy_(torch.triu(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")) +
                4 * torch.eye(n, dtype=torch.float64, device="cuda"))
        B0 = tq.empty(n, 4)
        B0.copy_(torch.randn(n, 4, generator=g, dtype=torch.float64, device="cuda"))
        B = tq.empty(n, 4)

        def run():
            B.copy_(B0)
            tq.trsm_lun(R, B)
        fl = 4.0 * n * n
    elif args.kernel == "tsmqr_tc":
        # tensor-core FP32 tsmqr ('L', 'C') on the same band as --kernel tsmqr --dtype f32
        import ctypes
        from tileqr import _lib
        w = ((n - NB) // 128) * 128
        dt = torch.float32
        A1, A2, V = tq.empty(NB, w, dtype=dt), tq.empty(NB, w, dtype=dt), tq.empty(NB, NB, dtype=dt)
        for t in (A1, A2):
            t.copy_(torch.randn(NB, w, generator=g, dtype=torch.float64, device="cuda"))
        V.copy_(torch.randn(NB, NB, generator=g, dtype=torch.float64, device="cuda") / 16)
        T = tq.empty(IB, NB, dtype=dt)
        T.copy_(torch.triu(torch.randn(IB, NB, generator=g, dtype=torch.float64, device="cuda")) / 16)
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        run = lambda: _lib.lib().tqr_stsmqr_tc(NB, w, NB, NB, P(A1), NB, P(A2), NB, P(V), NB, P(T), IB, P(err),
                                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        fl = 4.0 * NB * NB * w
    elif args.kernel == "tsmqr_wy":
        # the same band through the compact-WY form: one slot build for V and
        # T, then every 128-column chunk as three tensor-core products
        import ctypes
        from tileqr import _lib
        w = ((n - NB) // 128) * 128
        dt = torch.float32
        A1, A2, V = tq.empty(NB, w, dtype=dt), tq.empty(NB, w, dtype=dt), tq.empty(NB, NB, dtype=dt)
        for t in (A1, A2):
            t.copy_(torch.randn(NB, w, generator=g, dtype=torch.float64, device="cuda"))
        V.copy_(torch.randn(NB, NB, generator=g, dtype=torch.float64, device="cuda") / 16)
        T = tq.empty(IB, NB, dtype=dt)
        T.copy_(torch.triu(torch.randn(IB, NB, generator=g, dtype=torch.float64, device="cuda")) / 16)
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        nslot = _lib.lib().tqr_swy_slot_bytes()
        slot = torch.empty(nslot // 4, dtype=torch.float32, device="cuda")
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        run = lambda: _lib.lib().tqr_stsmqr_wy(NB, w, NB, NB, P(A1), NB, P(A2), NB, P(V), NB, P(T), IB, P(slot),
                                               nslot, P(err), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        fl = 4.0 * NB * NB * w
    elif args.kernel == "tsmqr":
        w = n - NB
        dt = torch.float32 if args.dtype == "f32" else torch.float64
        A1, A2, V = tq.empty(NB, w, dtype=dt), tq.empty(NB, w, dtype=dt), tq.empty(NB, NB, dtype=dt)
        for t in (A1, A2):
            t.copy_(torch.randn(NB, w, generator=g, dtype=torch.float64, device="cuda"))
        V.copy_(torch.randn(NB, NB, generator=g, dtype=torch.float64, device="cuda") / 16)
        T = tq.empty(IB, NB, dtype=dt)
        T.copy_(torch.triu(torch.randn(IB, NB, generator=g, dtype=torch.float64, device="cuda")) / 16)
        run = lambda: tq.tsmqr("L", "C", NB, w, NB, w, NB, IB, A1, A2, V, T, None)
        fl = 4.0 * NB * NB * w
    else:
        A1 = tq.empty(NB, NB)
        A2 = tq.empty(NB, NB)
        R0 = torch.triu(torch.randn(NB, NB, generator=g, dtype=torch.float64, device="cuda"))
        X0 = torch.randn(NB, NB, generator=g, dtype=torch.float64, device="cuda")
        T = tq.zeros(IB, NB)
        tau = torch.zeros(NB, dtype=torch.float64, device="cuda")

        def run():
            A1.copy_(R0 + 4 * torch.eye(NB, dtype=torch.float64, device="cuda"))
            A2.copy_(X0)
            if args.kernel == "tsqrt":
                tq.tsqrt(NB, NB, IB, A1, A2, T, tau, None)
            else:
                tq.geqrt(NB, NB, IB, A2, T, tau, None)
        fl = 2.0 * NB ** 3 if args.kernel == "tsqrt" else flops_square(NB)
    for _ in range(max(1, args.warmup)):
        run()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        run()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    res = {"kernel": args.kernel, "n": n, "ms": min(times), "tflops": fl / min(times) / 1e9,
           "all_ms": times}
    if args.dag_quantum is not None:
        res["dag_quantum"] = args.dag_quantum
    print(json.dumps(res), flush=True)
    return 0


def flops_square(n):
    return 4.0 / 3.0 * n ** 3


def config(n, N):
    return {"workload": f"flat-tree tile QR, {n}x{n} float64, nb={NB}, ib={IB}, entries N(0,1)",
            "m": n, "n": n, "nb": NB, "ib": IB, "parallelism": f"replicas x{N}",
            "l2": "inputs larger than L2 (A is 8 n^2 bytes, restored from a pristine copy each step)"}


# ---------------------------------------------------------------------------
# CPU side: the oracle (C restatement of NextLA's kernels, flat-tree driver)
# with its products in the host BLAS, as NextLA's larfb! runs them through
# LinearAlgebra.mul! on CPU arrays; the BLAS threads over the trailing
# columns of each panel (every host thread).  One step is the whole
# 8192^2 workload.
# ---------------------------------------------------------------------------
# tiles per flat group of the hierarchical tall-skinny QR (a sweep at 65536 x 512
# over 1, 2, 4, 8, 16, 32 measured 50.7, 45.2, 42.1, 42.2, 43.0, 50.7 ms)
HQR_GRP = 4


def cpu_sample_tflops(n, reps=1):
    """The oracle's flat-tree tile QR of the n x n N(0,1) workload (host BLAS
    products), timed on the host; returns (best TFLOP/s, seconds per run)."""
    import numpy as np
    import oracle
    oracle.build()
    rng = np.random.default_rng(SEED)
    A0 = np.asfortranarray(rng.standard_normal((n, n)))
    A = np.empty_like(A0, order="F")
    times = []
    with oracle.host_blas():
        for _ in range(reps):
            A[...] = A0
            t0 = time.perf_counter()
            oracle.tile_geqrf(A, NB, IB)
            times.append(time.perf_counter() - t0)
    return flops_square(n) / min(times) / 1e12, times


def cpu_cores_line():
    """Host cores and the BLAS thread count the CPU leg runs with."""
    import oracle
    threads = oracle.blas_threads() or cpu_threads()
    return threads, (f"{cpu_threads()} host cores, {threads} BLAS threads (scipy's OpenBLAS); the serial "
                     f"panel steps (NextLA's single-work-item geqr2/tsqrt block kernels) on one thread")


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
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
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference arm: NextLA's algorithm on the host cores (the oracle port,
    all host threads) on a bounded sample of the same workload."""
    if rank != 0:
        return 0
    import numpy as np
    import oracle
    oracle.build()
    threads, cores_note = cpu_cores_line()
    n = args.n
    rng = np.random.default_rng(SEED)
    A0 = np.asfortranarray(rng.standard_normal((n, n)))
    A = np.empty_like(A0, order="F")
    times = []
    with oracle.host_blas():
        # one untimed run loads the BLAS and pages the matrices in (a CPU run
        # has nothing else to warm up; more would only lengthen the arm)
        for _ in range(min(args.warmup, 1)):
            A[...] = A0
            oracle.tile_geqrf(A, NB, IB)
        for _ in range(args.steps):
            A[...] = A0
            t0 = time.perf_counter()
            oracle.tile_geqrf(A, NB, IB)
            times.append(time.perf_counter() - t0)
    total = sum(times)
    value = flops_square(n) * len(times) / total / 1e12
    sample = (f"the whole workload each step: flat-tree tile QR of the {n}x{n} N(0,1) float64 matrix "
              f"(nb={NB}, ib={IB}); {cores_note}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic N(0,1), seeded", "config": config(args.n, args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("Julia (the reference's language) is not installed on this host; the reference "
                 "arm runs the C restatement of NextLA's kernels (oracle/nextla_oracle.c) with its "
                 "larfb!/parfb! products in the host BLAS, as NextLA's mul! runs them on CPU arrays"),
    }
    print(json.dumps(line), flush=True)
    return 0


def haar(m, n, g, torch):
    """Haar-distributed m x n Q: this library's tile QR of a Gaussian matrix,
    Q formed by the Q application, columns signed by diag(R) > 0 (no
    dependency on torch.linalg, which cannot be loaded under the profiler)."""
    import tileqr as tq
    Z = tq.empty(m, n)
    Z.copy_(torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda"))
    T, _ = tq.tile_geqrf(Z, NB, IB)
    Q = tq.zeros(m, n)
    Q.diagonal().fill_(1.0)
    tq.tile_unmqr("N", Z, T, Q, NB, IB)
    torch.cuda.synchronize()
    return Q * torch.sign(torch.diagonal(Z)).unsqueeze(0)


def ls_problem(m, n, k, torch, seed=SEED):
    """The mixed-precision least-squares configuration: Float32-stored
    A = U diag(sigma) V^T (Haar U, V; sigma geometric from 1 to 1e-6),
    b = A x_true + 1e-10 N(0,1), k right-hand sides (synthetic, seeded)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    U = haar(m, n, g, torch)
    V = haar(n, n, g, torch)
    sigma = torch.logspace(0, -6, n, dtype=torch.float64, device="cuda")
    A = ((U * sigma.unsqueeze(0)) @ V.t()).float()
    del U, V
    x_true = torch.randn(n, k, generator=g, dtype=torch.float64, device="cuda")
    b = A.double() @ x_true + 1e-10 * torch.randn(m, k, generator=g, dtype=torch.float64, device="cuda")
    return A, b


def ls_bench(tq, torch, m=32768, n=4096, k=4, steps=2, warmup=1, orth=True):
    """Plain FP64 GPU least squares (FP64 tile QR, Q^T b, R x = c) against the
    mixed solve (FP32 tile QR + FP64 CGLS refinement) on the same problem."""
    A32, b = ls_problem(m, n, k, torch)
    A64 = A32.double()
    Ac = tq.empty(m, n, dtype=torch.float32)
    Ac.copy_(A32)
    bc = tq.empty(m, k)
    bc.copy_(b)
    Af = tq.empty(m, n)
    Bf = tq.empty(m, k)
    st = torch.cuda.current_stream()

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        out = fn()
        e1.record(st)
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    t64, tmx = [], []
    for rep in range(warmup + steps):
        Af.copy_(A64)
        Bf.copy_(b)
        torch.cuda.synchronize()
        X64, ms = timed(lambda: tq.lstsq_fp64(Af, Bf, NB, IB))
        if rep >= warmup:
            t64.append(ms)
        (Xm, it, rr), ms = timed(lambda: tq.lstsq_mixed(Ac, bc, NB, IB, maxit=60, tol=1e-13))
        if rep >= warmup:
            tmx.append(ms)
            phases = tq.dsgels_phases()
    X64 = X64.clone()
    normA = 1.0   # sigma_max = 1 by construction

    def berr(x):
        r = b - A64 @ x
        nb_ = (torch.linalg.norm(r, dim=0) / (normA * torch.linalg.norm(x, dim=0) +
                                              torch.linalg.norm(b, dim=0))).max().item()
        ls_ = (torch.linalg.norm(A64.t() @ r, dim=0) / (normA * torch.linalg.norm(r, dim=0))).max().item()
        return nb_, ls_

    be64, ls64 = berr(X64)
    bem, lsm = berr(Xm)
    res = {"workload": f"least squares, Float32-stored {m}x{n} A = U diag(sigma) V^T, sigma geometric "
                       f"1..1e-6, b = A x_true + 1e-10 N(0,1), {k} RHS",
           "fp64_ms": min(t64), "mixed_ms": min(tmx), "speedup": min(t64) / min(tmx),
           "mixed_iterations": it, "mixed_relres": rr, "mixed_phases_ms": phases,
           "normwise_backward_error_fp64": be64, "normwise_backward_error_mixed": bem,
           "ls_backward_error_fp64": ls64, "ls_backward_error_mixed": lsm,
           "rel_diff_mixed_vs_fp64": (torch.linalg.norm(Xm - X64) / torch.linalg.norm(X64)).item(),
           "note": ("normwise backward error ||b - Ax||/(||A|| ||x|| + ||b||) is bounded below by the "
                    "1e-10 noise for any least-squares solution; both forms reach the same value")}
    # the same solve on the flat tree (FP64 panels), for comparison
    oldg = tq.dsgels_hqr_group(0)
    try:
        tfl = []
        for rep in range(warmup + steps):
            (Xf, itf, _), ms = timed(lambda: tq.lstsq_mixed(Ac, bc, NB, IB, maxit=60, tol=1e-13))
            if rep >= warmup:
                tfl.append(ms)
                phf = tq.dsgels_phases()
        res["flat_tree"] = {"mixed_ms": min(tfl), "iterations": itf, "qr32_ms": phf["qr32_ms"],
                            "rel_diff_vs_fp64": (torch.linalg.norm(Xf - X64) / torch.linalg.norm(X64)).item()}
    finally:
        tq.dsgels_hqr_group(oldg)
    res["schedule"] = (f"hierarchical tree, groups of {oldg} tiles" if oldg and m // NB >= 2 * oldg
                       else "flat tree")
    # the same solve with the FP32 panels, for comparison (time, iterations)
    old = tq.dsgels_fp64_panels(False)
    try:
        t32 = []
        for rep in range(warmup + steps):
            (Xp, it32, rr32), ms = timed(lambda: tq.lstsq_mixed(Ac, bc, NB, IB, maxit=60, tol=1e-13))
            if rep >= warmup:
                t32.append(ms)
        res["fp32_panels"] = {"mixed_ms": min(t32), "iterations": it32,
                              "rel_diff_vs_fp64": (torch.linalg.norm(Xp - X64) / torch.linalg.norm(X64)).item()}
    finally:
        tq.dsgels_fp64_panels(old)
    if orth:
        # ||I - Q^T Q||_F of each stored factor, Q formed in FP64 from its V and T
        # (widened), so the figure is the factor's own, not an FP32 Q formation's
        def orth_of(F, T):
            Fd, Td = tq.empty(m, n), tq.empty(*T.shape)
            Fd.copy_(F.double())
            Td.copy_(T.double())
            Q = tq.zeros(m, n)
            Q.diagonal().fill_(1.0)
            tq.tile_unmqr("N", Fd, Td, Q, NB, IB)
            o = torch.linalg.norm(Q.t() @ Q - torch.eye(n, dtype=torch.float64, device="cuda")).item()
            del Fd, Td, Q
            return o
        for tag in ("mixed_flat", "mixed_fp32_panels", "fp64"):
            dt = torch.float64 if tag == "fp64" else torch.float32
            F = tq.empty(m, n, dtype=dt)
            F.copy_(A32 if dt == torch.float32 else A64)
            if tag == "mixed_flat":
                T, _ = tq.tile_geqrf_f64p(F, NB, IB)
            else:
                T, _ = tq.tile_geqrf(F, NB, IB)
            res[f"orth_I_minus_QtQ_fro_{tag}"] = orth_of(F, T)
            del F, T
        # the factor the default mixed solve uses: the hierarchical tree
        grp = tq.dsgels_hqr_group(0)
        tq.dsgels_hqr_group(grp)
        if grp and m // NB >= 2 * grp:
            F = tq.empty(m, n, dtype=torch.float32)
            F.copy_(A32)
            T, _, T2, _ = tq.tile_geqrf_tree(F, NB, IB, grp=grp, f64p=True)
            Fd, Td, T2d = tq.empty(m, n), tq.empty(*T.shape), tq.empty(*T2.shape)
            Fd.copy_(F.double())
            Td.copy_(T.double())
            T2d.copy_(T2.double())
            Q = tq.zeros(m, n)
            Q.diagonal().fill_(1.0)
            tq.tile_unmqr_tree("N", Fd, Td, T2d, Q, NB, IB, grp=grp)
            res["orth_I_minus_QtQ_fro_mixed"] = torch.linalg.norm(
                Q.t() @ Q - torch.eye(n, dtype=torch.float64, device="cuda")).item()
            del F, T, T2, Fd, Td, T2d, Q
        else:
            res["orth_I_minus_QtQ_fro_mixed"] = res["orth_I_minus_QtQ_fro_mixed_flat"]
    return res


def batched_bench(torch, nprob=4096, steps=5, warmup=3, peak=None, tune=True):
    """Batched uneven QR + least squares: nprob problems, m ~ U[32,512],
    n ~ U[16,m], k ~ U[1,8], N(0,1) entries, one persistent launch replayed
    from a CUDA graph.  Per precision: problems/s with inputs resident
    (device restore of the packed A, B outside the events, replay timed) and
    end to end (pinned host A, B copied in, replay, X copied out, all timed),
    plus the per-problem residual ||A^T(B - AX)|| / (||A|| (||A|| ||X|| + ||B||))."""
    from tileqr import _lib
    from tileqr import batched as Bt
    st = torch.cuda.current_stream()
    out = {"workload": (f"{nprob} independent least-squares problems, m ~ U[32,512], n ~ U[16,m], "
                        f"k ~ U[1,8] right-hand sides, N(0,1) entries (seeded); one persistent "
                        f"launch per batch, replayed from a CUDA graph"),
           "unit": "problems/s"}
    ms_, ns_, ks_ = Bt.random_sizes(nprob, seed=SEED % 1000)
    for tag, dt in (("f64", torch.float64), ("f32", torch.float32)):
        bg = Bt.BatchedGels(ms_, ns_, ks_, dtype=dt, tune=tune)
        g = torch.Generator(device="cuda").manual_seed(SEED)
        A0 = torch.randn(bg.A.shape, generator=g, device="cuda", dtype=torch.float64).to(dt)
        B0 = torch.randn(bg.B.shape, generator=g, device="cuda", dtype=torch.float64).to(dt)
        bg.capture()
        times = []
        launches0 = _lib.launch_count()
        for rep in range(warmup + steps):
            bg.A.copy_(A0)
            bg.B.copy_(B0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            bg.replay(sync=False)
            e1.record(st)
            torch.cuda.synchronize()
            if rep >= warmup:
                times.append(e0.elapsed_time(e1))
        launches = _lib.launch_count() - launches0
        bad = bg.status()
        res = bg.residuals(A0, B0)
        # end to end: pinned host buffers in, replay, X out
        hA = A0.cpu().pin_memory()
        hB = B0.cpu().pin_memory()
        hX = torch.empty_like(hB).pin_memory()
        ets = []
        for rep in range(1 + min(steps, 3)):
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(st)
            bg.A.copy_(hA, non_blocking=True)
            bg.B.copy_(hB, non_blocking=True)
            bg.replay(sync=False)
            hX.copy_(bg.B, non_blocking=True)
            f1.record(st)
            torch.cuda.synchronize()
            if rep >= 1:
                ets.append(f0.elapsed_time(f1))
        esz = A0.element_size()
        ms = statistics.median(times)
        fl = bg.flops()
        # algorithmic bytes: read A and B, write R and X: sum(mn + mk + n^2 + nk) elements
        abytes = esz * sum(int(m_) * int(n_) + int(m_) * int(k_) + int(n_) * int(n_) + int(n_) * int(k_)
                           for m_, n_, k_ in zip(ms_, ns_, ks_))
        hbm, hsrc = hbm_peak_gbs()
        out[tag] = {
            "problems_per_s": nprob / (ms / 1e3), "ms_per_batch": ms, "ms_min": min(times),
            "tflops": fl / (ms / 1e3) / 1e12, "algorithmic_flops_per_batch": fl,
            "frac_of_fp64_simt_peak": (fl / (ms / 1e3) / 1e12 / peak) if (peak and tag == "f64") else None,
            "algorithmic_bytes_per_batch": abytes, "hbm_gbs": abytes / ms / 1e6,
            "frac_of_hbm": abytes / ms / 1e6 / hbm, "hbm_peak_source": hsrc,
            "gpu_launches_per_batch": launches / (warmup + steps),
            "rejected_descriptors": bad[0],
            "residual_max": float(res.max().item()), "residual_median": float(res.median().item()),
            "e2e": {"value": nprob / (statistics.median(ets) / 1e3), "unit": "problems/s",
                    "ms_per_batch": statistics.median(ets),
                    "h2d_bytes_per_step": esz * (A0.numel() + B0.numel()),
                    "d2h_bytes_per_step": esz * B0.numel()},
            "tuning_ib_nw_by_n_class": {c: Bt.tuning(dt, c) for c in (32, 64, 128, 256, 512)},
        }
        bg.close()
        del bg, A0, B0, hA, hB, hX
    return out


def batched_sharded_bench(torch, nprob, world, rank, steps=5, warmup=3):
    """The FP64 batch of batched_bench split across the ranks by cost
    (tileqr.batched.shard): each rank solves its part in one persistent
    launch; time = max over ranks of the timed replays; no collective on the
    data path (results would be gathered on the host)."""
    from tileqr import batched as Bt
    ms_, ns_, ks_ = Bt.random_sizes(nprob, seed=SEED % 1000)
    mine = Bt.shard(ms_, ns_, ks_, world, rank)
    bg = Bt.BatchedGels(ms_[mine], ns_[mine], ks_[mine], dtype=torch.float64, tune=True)
    g = torch.Generator(device="cuda").manual_seed(SEED + rank)
    A0 = torch.randn(bg.A.shape, generator=g, device="cuda", dtype=torch.float64)
    B0 = torch.randn(bg.B.shape, generator=g, device="cuda", dtype=torch.float64)
    bg.capture()
    st = torch.cuda.current_stream()
    for _ in range(warmup):
        bg.A.copy_(A0)
        bg.B.copy_(B0)
        bg.replay(sync=True)
    total = 0.0
    for _ in range(steps):
        bg.A.copy_(A0)
        bg.B.copy_(B0)
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        bg.replay(sync=False)
        e1.record(st)
        torch.cuda.synchronize()
        total += reduce_max(e0.elapsed_time(e1), world)
    ms = total / steps
    cost = Bt.problem_cost(ms_, ns_, ks_)
    bad = bg.status()
    bg.close()
    return {"workload": f"{nprob} FP64 least-squares problems (the batched_uneven_gels batch) split by cost over "
                        f"{world} ranks", "problems_per_s": nprob / (ms / 1e3), "ms_per_batch": ms,
            "rank0_problems": int(mine.size), "rank0_cost_share": float(cost[mine].sum() / cost.sum()),
            "rejected_descriptors_rank0": bad[0], "scaling": "strong (fixed batch)"}


def adjoint_sharded_bench(torch, world, rank, batch=256, m=2048, n=256, steps=3, warmup=3):
    """The differentiable-QR batch split across the ranks (equal problems:
    tileqr.batched.shard gives each rank batch/world of them); forward and
    adjoint kernels with seeded cotangents, time = max over ranks."""
    import numpy as np
    from tileqr import autodiff as AD
    from tileqr import batched as Bt
    ones = np.ones(batch, dtype=np.int32)
    mine = Bt.shard(ones * m, ones * n, ones, world, rank)
    g = torch.Generator(device="cuda").manual_seed(SEED + rank)
    A = torch.randn((batch, m, n), generator=g, dtype=torch.float64, device="cuda")[torch.as_tensor(mine)]
    dQ = torch.randn((len(mine), m, n), generator=g, dtype=torch.float64, device="cuda")
    dR = torch.triu(torch.randn((len(mine), n, n), generator=g, dtype=torch.float64, device="cuda"))
    st = torch.cuda.current_stream()
    total = 0.0
    for rep in range(warmup + steps):
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        Q, R, F, tau = AD.qr_forward(A)
        AD.qr_backward(F, tau, dQ, dR)
        e1.record(st)
        torch.cuda.synchronize()
        t = reduce_max(e0.elapsed_time(e1), world)
        if rep >= warmup:
            total += t
    ms = total / steps
    return {"workload": f"differentiable QR forward + adjoint kernels, {batch} Float64 {m}x{n} problems split over "
                        f"{world} ranks", "problems_per_s": batch / (ms / 1e3), "ms_per_step": ms,
            "rank0_problems": int(len(mine)), "scaling": "strong (fixed batch)"}


def tall_bench(tq, torch, m=65536, n=512, steps=3, warmup=2, peak=None, dtype="f64"):
    """Tall-skinny tile QR (m x n, N(0,1), nb = 256, ib = 32): the flat-tree
    persistent kernel against the binary-tree driver (geqrt on every tile,
    ttqrt/ttmqr merges), flops 2mn^2 - 2n^3/3 per factorisation."""
    dt = torch.float64 if dtype == "f64" else torch.float32
    g = torch.Generator(device="cuda").manual_seed(SEED)
    A0 = tq.empty(m, n, dtype=dt)
    A0.copy_(torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda"))
    A = tq.empty(m, n, dtype=dt)
    st = torch.cuda.current_stream()
    flops = 2.0 * m * n * n - 2.0 * n ** 3 / 3

    def timed(fn):
        ts = []
        for rep in range(warmup + steps):
            A.copy_(A0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize()
            if rep >= warmup:
                ts.append(e0.elapsed_time(e1))
        return min(ts)

    t_flat = timed(lambda: tq.tile_geqrf(A, NB, IB))
    t_stream = timed(lambda: tq.tile_geqrf_tree(A, NB, IB, dag=False))
    t_tree = timed(lambda: tq.tile_geqrf_tree(A, NB, IB))
    t_hqr = timed(lambda: tq.tile_geqrf_tree(A, NB, IB, grp=HQR_GRP))
    out = {"workload": f"tall-skinny tile QR {m}x{n} {dtype} N(0,1), nb={NB}, ib={IB}",
           "flops": flops, "flat_dag_ms": t_flat, "tree_stream_ms": t_stream, "tree_ms": t_tree,
           "hqr_ms": t_hqr, "hqr_group": HQR_GRP,
           "flat_dag_tflops": flops / t_flat / 1e9, "tree_stream_tflops": flops / t_stream / 1e9,
           "tree_tflops": flops / t_tree / 1e9, "hqr_tflops": flops / t_hqr / 1e9,
           "speedup_tree_vs_flat": t_flat / t_tree, "speedup_hqr_vs_flat": t_flat / t_hqr,
           "tree": "binary reduction tree, one persistent launch over its task graph",
           "hqr": (f"hierarchical: groups of {HQR_GRP} tiles reduced flat into their leader, the leaders "
                   "by the binary tree, one persistent launch")}
    if peak and dtype == "f64":
        out["tree_frac_of_fp64_simt_peak"] = flops / t_tree / 1e9 / peak
        out["hqr_frac_of_fp64_simt_peak"] = flops / t_hqr / 1e9 / peak
    # the HBM view: A must be read and written at least once per pass, and the
    # factorisation needs two passes over it (panel reduction, then the update)
    hbm, src = hbm_peak_gbs()
    min_bytes = 2 * 2 * m * n * A.element_size()
    t_best = min(t_tree, t_hqr)
    out["hbm_min_bytes"] = min_bytes
    out["best_hbm_gbs_at_min_bytes"] = min_bytes / t_best / 1e6
    out["best_frac_of_hbm"] = min_bytes / t_best / 1e6 / hbm
    out["hbm_peak_gbs"] = hbm
    out["hbm_peak_source"] = src
    return out


def complex_bench(tq, torch, n=4096, steps=3, warmup=3, peak=None):
    """ComplexF64 and ComplexF32 tile QR of an n x n matrix (real and
    imaginary parts N(0,1), nb = 256, ib = 32) through the persistent kernel,
    against the stream driver.  Flops in real arithmetic: 4 x (4/3 n^3), the
    complex multiply-add being 8 real flops (4 fused multiply-adds)."""
    flops = 4.0 * 4.0 / 3.0 * n ** 3
    st = torch.cuda.current_stream()
    out = {"workload": f"complex tile QR {n}x{n}, N(0,1) real and imaginary parts, nb={NB}, ib={IB}",
           "flops": flops}
    for name, dt in (("c128", torch.complex128), ("c64", torch.complex64)):
        g = torch.Generator(device="cuda").manual_seed(SEED)
        A0 = tq.empty(n, n, dtype=dt)
        A0.copy_(torch.complex(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"),
                               torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda")).to(dt))
        A = tq.empty(n, n, dtype=dt)
        for mode, dag in (("dag", True), ("stream", False)):
            ts = []
            for rep in range(warmup + steps):
                A.copy_(A0)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(st)
                tq.tile_geqrf(A, NB, IB, dag=dag)
                e1.record(st)
                torch.cuda.synchronize()
                if rep >= warmup:
                    ts.append(e0.elapsed_time(e1))
            t = min(ts)
            out[f"{name}_{mode}_ms"] = t
            out[f"{name}_{mode}_tflops"] = flops / t / 1e9
        if peak and name == "c128":
            out["c128_dag_frac_of_fp64_simt_peak"] = flops / out["c128_dag_ms"] / 1e9 / peak
    return out


def hbm_peak_gbs():
    """The measured copy bandwidth of the GB300s (MEASURED_PEAKS.json)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def latency_bench(tq, torch, n=1024, nrhs=16, reps=20, warmup=5):
    """1024 x 1024 FP64 tile QR (U[-1,1], seeded, nb = 256, ib = 32: 4 x 4
    tiles) followed by Q^T applied to 1024 x 16 right-hand sides -- a
    latency-bound size, reported as latency: device time with the inputs
    resident, and end to end through the API from pinned host buffers (A and
    B in, R/V, T and Q^T B out)."""
    g = torch.Generator(device="cuda").manual_seed(SEED)
    A0 = tq.empty(n, n)
    A0.copy_(torch.rand(n, n, generator=g, dtype=torch.float64, device="cuda") * 2 - 1)
    B0 = tq.empty(n, nrhs)
    B0.copy_(torch.rand(n, nrhs, generator=g, dtype=torch.float64, device="cuda") * 2 - 1)
    A, B = tq.empty(n, n), tq.empty(n, nrhs)
    ts, taus = tq.tile_shapes(n, n, NB, IB)
    T, tau = tq.zeros(*ts), tq.zeros(*taus)
    st = torch.cuda.current_stream()

    def run():
        tq.tile_geqrf(A, NB, IB, T, tau)
        tq.tile_unmqr("C", A, T, B, NB, IB)

    qr_ms, all_ms = [], []
    for rep in range(warmup + reps):
        A.copy_(A0)
        B.copy_(B0)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(st)
        tq.tile_geqrf(A, NB, IB, T, tau)
        ev[1].record(st)
        tq.tile_unmqr("C", A, T, B, NB, IB)
        ev[2].record(st)
        torch.cuda.synchronize()
        if rep >= warmup:
            qr_ms.append(ev[0].elapsed_time(ev[1]))
            all_ms.append(ev[0].elapsed_time(ev[2]))
    hA = A0.t().cpu().pin_memory()
    hB = B0.t().cpu().pin_memory()
    hOut, hBo = torch.empty_like(hA).pin_memory(), torch.empty_like(hB).pin_memory()
    hT = torch.empty((ts[1], ts[0]), dtype=torch.float64).pin_memory()
    e2e = []
    for rep in range(warmup + reps):
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(st)
        A.t().copy_(hA, non_blocking=True)
        B.t().copy_(hB, non_blocking=True)
        run()
        hOut.copy_(A.t(), non_blocking=True)
        hT.copy_(T.t(), non_blocking=True)
        hBo.copy_(B.t(), non_blocking=True)
        f1.record(st)
        torch.cuda.synchronize()
        if rep >= warmup:
            e2e.append(f0.elapsed_time(f1))
    fl = flops_square(n) + 4.0 * n * n * nrhs - 2.0 * n * n * nrhs
    return {"workload": f"tile QR of a {n}x{n} U[-1,1] FP64 matrix (nb={NB}, ib={IB}) + Q^T on {n}x{nrhs}",
            "qr_ms_median": statistics.median(qr_ms), "qr_plus_apply_ms_median": statistics.median(all_ms),
            "qr_plus_apply_ms_min": min(all_ms), "e2e_ms_median": statistics.median(e2e),
            "flops": fl, "tflops_at_median": fl / statistics.median(all_ms) / 1e9,
            "h2d_bytes": 8 * (n * n + n * nrhs), "d2h_bytes": 8 * (n * n + ts[0] * ts[1] + n * nrhs),
            "bound": "latency (16 tiles: the panel chain of 4 geqrt + 6 tsqrt is the critical path)"}


def autotune_square(tq, torch, n, candidates=((256, 32), (256, 16), (256, 64), (128, 32), (128, 16)),
                    steps=2, warmup=1):
    """The square FP64 tile QR over a few (nb, ib) tilings: ms and TFLOP/s of
    each (persistent kernel where the tiling allows it), and the best."""
    g = torch.Generator(device="cuda").manual_seed(SEED)
    A0 = tq.empty(n, n)
    A0.copy_(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
    A = tq.empty(n, n)
    st = torch.cuda.current_stream()
    res = {}
    for nb, ib in candidates:
        ts, taus = tq.tile_shapes(n, n, nb, ib)
        T, tau = tq.zeros(*ts), tq.zeros(*taus)
        times = []
        for rep in range(warmup + steps):
            A.copy_(A0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            tq.tile_geqrf(A, nb, ib, T, tau)
            e1.record(st)
            torch.cuda.synchronize()
            if rep >= warmup:
                times.append(e0.elapsed_time(e1))
        t = min(times)
        res[f"nb{nb}_ib{ib}"] = {"ms": t, "tflops": flops_square(n) / t / 1e9,
                                 "persistent": tq.dag_worksize(n, n, nb, ib) is not None}
        del T, tau
    best = max(res, key=lambda k: res[k]["tflops"])
    # the library's own tuner (tqr_tile_autotune) on the same shape
    t0 = time.perf_counter()
    lnb, lib_ib = tq.autotune_tiling(n, n, torch.float64)
    lib = {"nb": lnb, "ib": lib_ib, "tune_s": time.perf_counter() - t0}
    return {"workload": f"tile QR {n}x{n} FP64 N(0,1), (nb, ib) sweep", "results": res, "best": best,
            "library_autotune": lib}


def lapack_dgeqrf_tflops(n):
    """scipy's LAPACK dgeqrf (OpenBLAS, all host threads) on an n x n N(0,1)
    matrix: the library CPU QR beside the restated reference algorithm."""
    import numpy as np
    from scipy.linalg import lapack
    rng = np.random.default_rng(SEED)
    A = np.asfortranarray(rng.standard_normal((n, n)))
    t0 = time.perf_counter()
    _, _, _, info = lapack.dgeqrf(A, overwrite_a=1)
    dt = time.perf_counter() - t0
    return flops_square(n) / dt / 1e12, dt


def adjoint_kernels_complex(torch, batch, m, n, steps, warmup, dtype):
    """Forward and adjoint kernels of the complex differentiable QR on a batch
    of complex N(0,1) problems with seeded cotangents, CUDA-event timed on the
    launching stream.  Flops are real flops: 4x the real counts for a complex
    multiply-add (factorisation 4 (2mn^2 - 2n^3/3), explicit Q 4 (2mn^2 - 2n^3/3))."""
    from tileqr import autodiff as AD
    tdt = {"c128": torch.complex128, "c64": torch.complex64}[dtype]
    st = torch.cuda.current_stream()
    g = torch.Generator(device="cuda").manual_seed(SEED)

    def cr(*s):
        return torch.complex(torch.randn(s, generator=g, dtype=torch.float64, device="cuda"),
                             torch.randn(s, generator=g, dtype=torch.float64, device="cuda")).to(tdt)

    A, Qb, Rb = cr(batch, m, n), cr(batch, m, n), torch.triu(cr(batch, n, n))
    fwd_ms, bwd_ms = [], []
    for rep in range(warmup + steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(st)
        Q, R, F, tau = AD.qr_forward(A)
        e[1].record(st)
        Ab = AD.qr_backward(F, tau, Qb, Rb)
        e[2].record(st)
        torch.cuda.synchronize()
        if rep >= warmup:
            fwd_ms.append(e[0].elapsed_time(e[1]))
            bwd_ms.append(e[1].elapsed_time(e[2]))
    finite = bool(torch.isfinite(torch.view_as_real(Ab)).all())
    f_fwd = batch * 4.0 * 2 * (2.0 * m * n * n - 2.0 * n ** 3 / 3.0)
    fm, bm = statistics.median(fwd_ms), statistics.median(bwd_ms)
    return {"workload": f"QR forward and adjoint kernels, batch of {batch} {dtype} {m}x{n}, seeded cotangents",
            "fwd_ms": fm, "bwd_ms": bm, "fwd_tflops_real": f_fwd / (fm * 1e-3) / 1e12, "finite": finite}


def adjoint_bench(torch, batch=256, m=2048, n=256, steps=3, warmup=3, peak=None, kernels_only=False,
                  dtype="f64"):
    """Differentiable QR: (Q, R) = qr(A) for a batch of 256 Float64 2048x256
    N(0,1) matrices, loss 1/2||R^-1 Q^T b - y||^2 + <dQ, Q> + <dR, R> with
    seeded b, y, dQ, dR, backward through the adjoint kernel.  Times the
    forward kernel, the backward kernel and the whole autograd step; checks
    one problem against the CPU FP64 reference adjoint and the whole batch
    against a central difference (h = 1e-6).  With kernels_only the element
    type may be complex ("c128", "c64": the forward and adjoint kernels on
    complex N(0,1) problems; real and imaginary parts seeded alike)."""
    import numpy as np

    if dtype != "f64":
        if not kernels_only:
            raise SystemExit("--dtype other than f64 needs --adjoint-kernels")
        return adjoint_kernels_complex(torch, batch, m, n, steps, warmup, dtype)
    import oracle
    from tileqr import _lib
    from tileqr import autodiff as AD
    st = torch.cuda.current_stream()
    g = torch.Generator(device="cuda").manual_seed(SEED)
    A = torch.randn((batch, m, n), generator=g, dtype=torch.float64, device="cuda")
    b = torch.randn((batch, m), generator=g, dtype=torch.float64, device="cuda")
    y = torch.randn((batch, n), generator=g, dtype=torch.float64, device="cuda")
    dQ = torch.randn((batch, m, n), generator=g, dtype=torch.float64, device="cuda")
    dR = torch.randn((batch, n, n), generator=g, dtype=torch.float64, device="cuda")

    def loss(Q, R):
        c = torch.einsum("bmn,bm->bn", Q, b)
        x = torch.linalg.solve_triangular(R, c.unsqueeze(-1), upper=True).squeeze(-1)
        return 0.5 * ((x - y) ** 2).sum() + (dQ * Q).sum() + (dR * torch.triu(R)).sum()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    fwd_ms, bwd_ms, step_ms = [], [], []
    launches0 = _lib.launch_count()
    for rep in range(warmup + steps):
        e0, e1, e2, e3 = ev(), ev(), ev(), ev()
        e0.record(st)
        Q, R, F, tau = AD.qr_forward(A)
        e1.record(st)
        if kernels_only:
            # the kernels alone (profiling): seeded cotangents instead of the loss's
            Qb, Rb = dQ, torch.triu(dR)
        else:
            Ql = Q.requires_grad_(True)
            Rl = R.requires_grad_(True)
            Qb, Rb = torch.autograd.grad(loss(Ql, Rl), (Ql, Rl))
        e2.record(st)
        Ab = AD.qr_backward(F, tau, Qb, Rb)
        e3.record(st)
        torch.cuda.synchronize()
        if rep >= warmup:
            fwd_ms.append(e0.elapsed_time(e1))
            bwd_ms.append(e2.elapsed_time(e3))
            step_ms.append(e0.elapsed_time(e3))
    launches = (_lib.launch_count() - launches0) / (warmup + steps)
    if kernels_only:
        return {"workload": f"QR forward and adjoint kernels, batch of {batch} Float64 {m}x{n}, seeded cotangents",
                "fwd_ms": statistics.median(fwd_ms), "bwd_ms": statistics.median(bwd_ms)}
    # the autograd path end to end (rule's backward) must give the same gradient
    Ar = A.detach().clone().requires_grad_(True)
    Q, R = AD.qr(Ar)
    loss(Q, R).backward()
    G = Ar.grad.detach()
    same = float((G - Ab).abs().max().item())
    # one problem against the CPU FP64 reference adjoint
    p = 0
    Qh, Rh = Q[p].detach().cpu().numpy(), R[p].detach().cpu().numpy()
    _, qb, rb = oracle.ls_loss_cotangents(Qh, Rh, b[p].cpu().numpy(), y[p].cpu().numpy(), dQ[p].cpu().numpy(),
                                          dR[p].cpu().numpy())
    Qo, Ro, _ = oracle.qr_explicit(A[p].cpu().numpy(), 256, 32)
    ref = oracle.qr_adjoint(Qo, Ro, qb, rb)
    rel_cpu = float(np.linalg.norm(G[p].cpu().numpy() - ref) / np.linalg.norm(ref))
    # central difference over the whole batch along one direction
    E = torch.randn(A.shape, generator=g, dtype=torch.float64, device="cuda")
    h = 1e-6
    with torch.no_grad():
        Qp, Rp, _, _ = AD.qr_forward(A + h * E)
        Qm, Rm, _, _ = AD.qr_forward(A - h * E)
        fd = (loss(Qp, Rp) - loss(Qm, Rm)).item() / (2 * h)
    an = (G * E).sum().item()
    f_fact = batch * (2.0 * m * n * n - 2.0 * n ** 3 / 3)        # factorisation
    f_q = batch * (2.0 * m * n * n - 2.0 * n ** 3 / 3)           # forming the thin Q
    f_bwd = batch * (5.0 * m * n * n + n ** 3 / 3.0)             # adjoint with an explicit Q
    fw, bw, sp = statistics.median(fwd_ms), statistics.median(bwd_ms), statistics.median(step_ms)
    return {
        "workload": (f"differentiable QR: batch of {batch} Float64 {m}x{n} N(0,1) matrices, loss "
                     f"1/2||R^-1 Q^T b - y||^2 + <dQ,Q> + <dR,R> (seeded b, y, dQ, dR); forward kernel "
                     f"(tile QR + explicit Q), autograd of the loss, adjoint kernel with T recomputed"),
        "fwd_ms": fw, "bwd_ms": bw, "step_ms": sp,
        "fwd_factorisation_tflops": f_fact / (fw / 1e3) / 1e12,
        "fwd_tflops_incl_q": (f_fact + f_q) / (fw / 1e3) / 1e12,
        "bwd_tflops_algorithmic": f_bwd / (bw / 1e3) / 1e12,
        "flop_counts": {"factorisation": f_fact, "form_q": f_q, "adjoint_explicit_q_count": f_bwd,
                        "note": ("the adjoint kernel applies Q through the compact reflectors "
                                 "(about 9 m n^2 flops per problem) instead of keeping Q; the "
                                 "algorithmic count is the 5 m n^2 of the explicit-Q formula")},
        "frac_of_fp64_simt_peak_fwd": ((f_fact + f_q) / (fw / 1e3) / 1e12 / peak) if peak else None,
        "gpu_launches_per_step": launches,
        "rel_err_vs_cpu_fp64_adjoint_problem0": rel_cpu,
        "central_difference": {"h": h, "fd": fd, "analytic": an, "rel_err": abs(fd - an) / abs(an)},
        "autograd_vs_direct_max_abs_diff": same,
    }


def fp64_peak(tq_lib, torch):
    """SIMT DFMA ceiling of this GPU (independent FMA chains), TFLOP/s."""
    import ctypes
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sms * 8, 20000
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        rc = tq_lib.lib().tqr_fp64_peak_probe(blocks, iters, ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(st.cuda_stream))
        e1.record(st)
        st.synchronize()
        if rc != 0:
            raise RuntimeError(f"fp64 probe failed: {rc}")
        ms = e0.elapsed_time(e1)
        best = max(best, 16.0 * iters * blocks * 256 / ms / 1e9)
    return best


def fp64_mma_peak(tq_lib, torch):
    """FP64 tensor-core (DMMA, mma.sync.m8n8k4.f64) rate of this GPU, and
    the DMMA/DFMA split when some warps of each CTA run one and the rest the
    other (tqr_fp64_mma_probe): whether the two FP64 paths add up."""
    import ctypes
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, iters = sms * 2, 4000
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    fa, fb = ctypes.c_double(0), ctypes.c_double(0)
    mix = {}
    for dw in (8, 0, 2, 4, 6, 8):
        best = None
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            rc = tq_lib.lib().tqr_fp64_mma_probe(blocks, iters, dw, ctypes.c_void_p(out.data_ptr()),
                                                ctypes.byref(fa), ctypes.byref(fb),
                                                ctypes.c_void_p(st.cuda_stream))
            e1.record(st)
            st.synchronize()
            if rc != 0:
                raise RuntimeError(f"fp64 mma probe failed: {rc}")
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        mix[f"dmma_warps_{dw}_of_8"] = {"dmma_tflops": fa.value / best / 1e9, "dfma_tflops": fb.value / best / 1e9,
                                        "total_tflops": (fa.value + fb.value) / best / 1e9}
    return mix["dmma_warps_8_of_8"]["dmma_tflops"], mix


def noalloc_vs_workspace(tq, torch, sizes=(4096, 8192), reps=3):
    """The allocation-free tile QR (tqr_dtile_geqrf_noalloc: schedule in a
    fixed device array, written on the device in buckets of key
    4 min(column, k + 1) + row)
    against the workspace entry point (critical-path order) on the same
    matrix."""
    import ctypes
    from tileqr import _lib
    st = torch.cuda.current_stream()
    out = {}
    for n in sizes:
        g = torch.Generator(device="cuda").manual_seed(SEED + n)
        A0 = tq.empty(n, n)
        A0.copy_(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
        A = tq.empty(n, n)
        ts, taus = tq.tile_shapes(n, n, NB, IB)
        T, tau = tq.zeros(*ts), tq.zeros(*taus)
        P = lambda t: ctypes.c_void_p(t.data_ptr())

        def noalloc():
            rc = _lib.lib().tqr_dtile_geqrf_noalloc(n, n, NB, IB, P(A), n, P(T), ts[0], P(tau), taus[0],
                                                   ctypes.c_void_p(st.cuda_stream))
            if rc != 0:
                raise RuntimeError(f"noalloc: {rc}")

        def workspace():
            tq.tile_geqrf(A, NB, IB, T, tau)

        res = {}
        for name, fn in (("workspace_ms", workspace), ("noalloc_ms", noalloc)):
            ts_ = []
            for rep in range(reps + 1):
                A.copy_(A0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                fn()
                e1.record(st)
                torch.cuda.synchronize()
                if rep:
                    ts_.append(e0.elapsed_time(e1))
            res[name] = min(ts_)
        status = ctypes.c_int(-1)
        _lib.lib().tqr_tile_noalloc_status(ctypes.byref(status), None, ctypes.c_void_p(st.cuda_stream))
        res["noalloc_status"] = status.value
        res["noalloc_over_workspace"] = res["noalloc_ms"] / res["workspace_ms"]
        out[f"{n}x{n}"] = res
        del A0, A, T, tau
    return out


def summaries(ls, bat, adj, tall, noalloc):
    """Short figures of the other configurations, placed last on the JSON line."""
    out = {}
    if ls:
        out["mixed_ls_32768x4096"] = {
            "speedup_vs_fp64": round(ls["speedup"], 2), "fp64_ms": round(ls["fp64_ms"], 1),
            "mixed_ms": round(ls["mixed_ms"], 1), "iters": ls["mixed_iterations"],
            "ls_berr_mixed": float(f"{ls['ls_backward_error_mixed']:.3e}"),
            "ls_berr_fp64": float(f"{ls['ls_backward_error_fp64']:.3e}"),
            "nw_berr_mixed": float(f"{ls['normwise_backward_error_mixed']:.4e}"),
            "nw_berr_fp64": float(f"{ls['normwise_backward_error_fp64']:.4e}"),
            "x_rel_to_fp64": float(f"{ls['rel_diff_mixed_vs_fp64']:.2e}")}
        if "orth_I_minus_QtQ_fro_mixed" in ls:
            out["mixed_ls_32768x4096"]["orth_mixed"] = float(f"{ls['orth_I_minus_QtQ_fro_mixed']:.2e}")
            out["mixed_ls_32768x4096"]["orth_fp32_panels"] = float(
                f"{ls['orth_I_minus_QtQ_fro_mixed_fp32_panels']:.2e}")
        if ls.get("flat_tree"):
            out["mixed_ls_32768x4096"]["flat_tree_ms_iters"] = [round(ls["flat_tree"]["mixed_ms"], 1),
                                                                ls["flat_tree"]["iterations"]]
            out["mixed_ls_32768x4096"]["schedule"] = ls.get("schedule")
        if ls.get("fp32_panels"):
            out["mixed_ls_32768x4096"]["fp32_panels_ms_iters"] = [round(ls["fp32_panels"]["mixed_ms"], 1),
                                                                  ls["fp32_panels"]["iterations"]]
    if bat:
        for tag in ("f64", "f32"):
            b = bat.get(tag)
            if b:
                out[f"batched_{tag}"] = {"problems_per_s": round(b["problems_per_s"]),
                                         "e2e_problems_per_s": round(b["e2e"]["value"]),
                                         "tflops": round(b["tflops"], 3), "residual_max": float(f"{b['residual_max']:.2e}")}
                if b.get("frac_of_fp64_simt_peak"):
                    out[f"batched_{tag}"]["frac_fp64_simt"] = round(b["frac_of_fp64_simt_peak"], 3)
    if adj and "fwd_ms" in adj:
        out["adjoint_256x2048x256"] = {"fwd_ms": round(adj["fwd_ms"], 1), "bwd_ms": round(adj["bwd_ms"], 1)}
        if adj.get("central_difference"):
            out["adjoint_256x2048x256"]["fd_rel_err"] = float(f"{adj['central_difference']['rel_err']:.2e}")
        if adj.get("rel_err_vs_cpu_fp64_adjoint_problem0") is not None:
            out["adjoint_256x2048x256"]["cpu_adjoint_rel_err"] = float(
                f"{adj['rel_err_vs_cpu_fp64_adjoint_problem0']:.2e}")
    if tall:
        out["tall_65536x512"] = {"hqr_ms": round(tall["hqr_ms"], 1), "flat_ms": round(tall["flat_dag_ms"], 1),
                                 "hqr_tflops": round(tall["hqr_tflops"], 3)}
    if noalloc:
        out["noalloc_over_workspace"] = {k: round(v["noalloc_over_workspace"], 3) for k, v in noalloc.items()}
    return out


def cublas_dgemm_tflops(torch, n=4096):
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    a @ b
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    a @ b
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * n ** 3 / e0.elapsed_time(e1) / 1e9


def main():
    args = parse()
    if args.kernel:
        return kernel_bench(args)
    if args.ls_only:
        import torch

        import tileqr as tq
        import tileqr_build
        tileqr_build.build()
        tq.set_blocking(False)
        res = ls_bench(tq, torch, args.ls_m, args.ls_n, 4, max(1, args.steps), max(1, args.warmup),
                       orth=not args.ls_no_orth)
        print(json.dumps(res), flush=True)
        return 0
    if args.tall_only:
        import torch

        import tileqr as tq
        import tileqr_build
        from tileqr import _lib
        tileqr_build.build()
        tq.set_blocking(False)
        peak = fp64_peak(_lib, torch)
        res = {"f64": tall_bench(tq, torch, peak=peak), "f32": tall_bench(tq, torch, dtype="f32")}
        print(json.dumps(res), flush=True)
        return 0
    if args.latency_only:
        import torch

        import tileqr as tq
        import tileqr_build
        tileqr_build.build()
        tq.set_blocking(False)
        print(json.dumps(latency_bench(tq, torch)), flush=True)
        return 0
    if args.complex_only:
        import torch

        import tileqr as tq
        import tileqr_build
        from tileqr import _lib
        tileqr_build.build()
        tq.set_blocking(False)
        res = complex_bench(tq, torch, args.complex_n, max(1, args.steps), max(3, args.warmup),
                            peak=fp64_peak(_lib, torch))
        print(json.dumps(res), flush=True)
        return 0
    if args.adjoint_only:
        import torch

        import tileqr_build
        from tileqr import _lib
        tileqr_build.build()
        ab, am, an = (int(v) for v in args.adjoint_shape.split(","))
        if (ab, am, an) != (256, 2048, 256) and not args.adjoint_kernels:
            raise SystemExit("--adjoint-shape needs --adjoint-kernels")
        res = adjoint_bench(torch, ab, am, an, max(1, args.steps), max(3, args.warmup),
                            kernels_only=args.adjoint_kernels,
                            peak=fp64_peak(_lib, torch), dtype=args.dtype)
        print(json.dumps(res), flush=True)
        return 0
    if args.batched_only:
        import torch

        import tileqr_build
        from tileqr import _lib
        tileqr_build.build()
        res = batched_bench(torch, args.batched_n, max(1, args.steps), max(3, args.warmup), tune=not args.batched_no_tune,
                            peak=fp64_peak(_lib, torch))
        print(json.dumps(res), flush=True)
        return 0
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        # host-only arm: rank 0 times the reference algorithm, other ranks exit
        # without work, so no process group (and no GPU) is needed
        return run_reference(args, world, rank)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    import torch

    import tileqr as tq
    import tileqr_build
    from tileqr import _lib

    tileqr_build.build()
    torch.cuda.set_device(local)
    tq.set_blocking(False)
    n = args.n
    flops = flops_square(n)
    g = torch.Generator(device="cuda").manual_seed(SEED + rank)
    A0 = tq.empty(n, n)
    A0.copy_(torch.randn(n, n, generator=g, dtype=torch.float64, device="cuda"))
    A = tq.empty(n, n)
    ts, taus = tq.tile_shapes(n, n, NB, IB)
    T = tq.zeros(*ts)
    tau = tq.zeros(*taus)
    st = torch.cuda.current_stream()

    def step():
        A.copy_(A0)
        tq.tile_geqrf(A, NB, IB, T, tau)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    clocks = Clocks(torch.cuda.current_device())
    clocks.start()
    _lib.profile_enable(True)
    _lib.profile_read()
    launches0 = _lib.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    barrier(world)
    launches = _lib.launch_count() - launches0
    _lib.profile_enable(False)
    prof_n, prof_ms, prof_flops = _lib.profile_read()
    clk = clocks.stop()
    dag = tq.dag_stats()
    ms_total = reduce_max(e0.elapsed_time(e1), world)
    ms_step = ms_total / args.steps
    value = flops * world * args.steps / (ms_total / 1e3) / 1e12

    # end to end through the public API: host buffers in, factor, host buffers out
    # (right after the timed region, before the peak probes below heat the GPU)
    e2e = None
    if not args.no_e2e:
        hA = torch.empty((n, n), dtype=torch.float64).pin_memory()
        hA.copy_(A0.t().cpu())
        hOut = torch.empty((n, n), dtype=torch.float64).pin_memory()
        hT = torch.empty((ts[1], ts[0]), dtype=torch.float64).pin_memory()
        Ad = tq.empty(n, n)

        phase_ev = []

        def e2e_step(record=False):
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)] if record else None
            if record:
                evs[0].record(st)
            Ad.t().copy_(hA, non_blocking=True)         # H2D of the input matrix
            if record:
                evs[1].record(st)
            tq.tile_geqrf(Ad, NB, IB, T, tau)
            if record:
                evs[2].record(st)
            hOut.copy_(Ad.t(), non_blocking=True)       # D2H of R and V
            hT.copy_(T.t(), non_blocking=True)          # D2H of T
            if record:
                evs[3].record(st)
                phase_ev.append(evs)
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        ks = max(1, min(args.steps, 3))
        eclk = Clocks(torch.cuda.current_device())
        eclk.start()
        barrier(world)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(st)
        marks = []
        for _ in range(ks):
            e2e_step(record=True)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(st)
            marks.append(ev)
        f1.record(st)
        torch.cuda.synchronize()
        ems = reduce_max(f0.elapsed_time(f1), world)
        steps_ms = [f0.elapsed_time(marks[0])] + [marks[q].elapsed_time(marks[q + 1]) for q in range(ks - 1)]
        e2e = {"value": flops * world * ks / (ems / 1e3) / 1e12, "unit": UNIT,
               "h2d_bytes_per_step": 8 * n * n, "d2h_bytes_per_step": 8 * n * n + 8 * ts[0] * ts[1],
               "steps": ks, "ms_per_step": ems / ks, "step_ms": steps_ms, "clocks": eclk.stop(),
               "phase_ms_median": {nm: statistics.median(e[q].elapsed_time(e[q + 1]) for e in phase_ev)
                                   for q, nm in enumerate(("h2d", "factor", "d2h"))}}

    # roofline of the dominant kernel (the one persistent launch per step)
    peak = fp64_peak(_lib, torch)
    mma_peak, mma_mix = fp64_mma_peak(_lib, torch)
    dgemm = cublas_dgemm_tflops(torch)
    achieved = (prof_flops / prof_n) / (prof_ms / prof_n) / 1e9 if prof_n else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    roofline = {"bound": "fp64_simt", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "fp64_mma_tflops": mma_peak,
                "frac_of_fp64_mma": (achieved / mma_peak) if (achieved and mma_peak) else None,
                "cublas_dgemm_tflops": dgemm,
                "fp64_mma_dfma_mix": mma_mix,
                "kernel": ("k_tile_dag (one persistent launch per factorisation: panel, unmqr and "
                           "tsmqr tasks), FP64 SIMT DFMA; algorithmic flops 4/3 n^3 per launch"),
                "peak_source": ("measured live: DFMA-chain probe (tqr_fp64_peak_probe), the FP64 ceiling "
                                "on this GPU; the FP64 tensor-core rate (tqr_fp64_mma_probe, "
                                "mma.sync.m8n8k4.f64) and cuBLAS DGEMM measured alongside; "
                                "MEASURED_PEAKS.json has no FP64 figure"),
                "timed_launches": prof_n, "algorithmic_flops_per_launch": (prof_flops / prof_n) if prof_n else None,
                "ms_per_launch": (prof_ms / prof_n) if prof_n else None}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads, cores_note = cpu_cores_line()
        v, times = cpu_sample_tflops(n, reps=2)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"the workload itself: oracle (C restatement of NextLA's kernels, larfb!/parfb! "
                          f"products in the host BLAS as NextLA's mul! does) flat-tree tile QR of the "
                          f"{n}x{n} N(0,1) matrix, nb={NB}, ib={IB}; best of {len(times)} runs "
                          f"({', '.join(f'{t:.1f}' for t in times)} s); {cores_note}")}
        try:
            lv, lt = lapack_dgeqrf_tflops(n)
            cpu["lapack_dgeqrf"] = {"value": lv, "unit": UNIT, "seconds": lt,
                                    "sample": f"scipy LAPACK dgeqrf (OpenBLAS, all host threads) on the {n}x{n} matrix"}
        except Exception as ex:       # scipy missing on the host: report why
            cpu["lapack_dgeqrf"] = {"unavailable": str(ex)[:200]}

    ls = None
    if rank == 0 and world == 1 and not args.no_ls:
        ls = ls_bench(tq, torch, args.ls_m, args.ls_n, 4, 2, 1, orth=not args.ls_no_orth)

    bat = None
    if rank == 0 and world == 1 and not args.no_batched:
        bat = batched_bench(torch, args.batched_n, 5, 3, peak=peak)

    tall = None
    if rank == 0 and world == 1 and not args.no_tall:
        tall = tall_bench(tq, torch, peak=peak)

    adj = None
    if rank == 0 and world == 1 and not args.no_adjoint:
        adj = adjoint_bench(torch, 256, 2048, 256, 3, 3, peak=peak)

    sharded = None
    if world > 1 and not args.no_batched:
        sharded = batched_sharded_bench(torch, args.batched_n, world, rank)
    adj_sharded = None
    if world > 1 and not args.no_adjoint:
        adj_sharded = adjoint_sharded_bench(torch, world, rank)

    cplx = None
    if rank == 0 and world == 1 and not args.no_complex:
        cplx = complex_bench(tq, torch, args.complex_n, 3, 3, peak=peak)

    lat = None
    tune = None
    noalloc = None
    if rank == 0 and world == 1 and not args.no_extras:
        lat = latency_bench(tq, torch)
        tune = autotune_square(tq, torch, n)
        noalloc = noalloc_vs_workspace(tq, torch)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic N(0,1), seeded", "config": config(n, world),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": launches,
            "dag_stats_last_step": dag,
            "complex_tile_qr": cplx,
            "latency_1024": lat,
            "tiling_sweep": tune,
            "noalloc_vs_workspace": noalloc,
            "batched_uneven_gels_sharded": sharded,
            "differentiable_qr_sharded": adj_sharded,
            "tall_skinny_65536x512": tall,
            "differentiable_qr": adj,
            "batched_uneven_gels": bat,
            "least_squares_mixed_vs_fp64": ls,
            # last on the line, so that a record keeping only the tail still has them
            "summary_other_configs": summaries(ls, bat, adj, tall, noalloc),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
