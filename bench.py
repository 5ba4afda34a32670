"""Benchmark: Lanczos H.psi throughput on the 4x4 Hubbard cluster at half
filling (16 sites, N=16, Sz=0, sector dimension 165,636,900, FP64 vectors).

A step is one Hamiltonian-vector product y <- y + H x of that sector (the
reference's mult_add, performed by every Lanczos / band-Lanczos iteration).
value = algorithmic bytes (24 B per basis state: read x, read y, write y)
x steps / device time, with both vectors (1.33 GB each, larger than L2)
resident in HBM.  e2e = the same metric through the public host API
(Hamiltonian.mult_add: x and y copied in from pinned host memory, y copied
back, every step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl qcmg|reference]

--impl reference times the CPU oracle's port of the reference's factorized
product (oracle/qcm_oracle.c) on the host cores with all threads.
Multi-GPU runs are independent replicas (the product does not shard).
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
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

METRIC = "lanczos_hpsi_gbs"
UNIT = "GB/s"
NX, NY = 4, 4
NEL = None  # electrons (None: half filling)
PARAMS = {"t": 1.0, "U": 8.0, "mu": 4.0}
BYTES_PER_STATE = 24


def sector_of(nx, ny):
    """(sector, n_up, n_dn): half filling, or NEL electrons when set."""
    n = NEL if NEL else nx * ny
    return f"R0:N{n}:S{n % 2}", (n + n % 2) // 2, n // 2


def workload_config(dim=165636900):
    sec = sector_of(NX, NY)[0]
    return {"workload": f"{NX}x{NY} Hubbard cluster, t=1 U=8 mu=4, sector {sec} "
                        f"(dim {dim:,}), y <- y + H x",
            "dim": dim, "bytes_per_step": BYTES_PER_STATE * dim,
            "l2": "inputs larger than L2", "parallelism": "replicas"}


def model_ops():
    from models import hubbard_cluster
    return hubbard_cluster(NX, NY)


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """Per-launch DRAM bytes of the product kernel from the committed ncu
    summary, or None."""
    p = os.path.join(ROOT, "profiles", "matvec_4x4_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch_full:"):
            return float(line.split(":")[1])
    return None


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()  # sampling is live before the timed region starts
            while not self.rows and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.rows)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        # rows taken before the timed region began are dropped, unless nothing else came
        rows = self.rows[getattr(self, "skip", 0):] or self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_port_timing(steps, threads):
    """Times the oracle's port of the reference's factorized product on the
    host (all `threads`), on the same sector; returns (GB/s, seconds/step)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import qcm_oracle as qo
    ns, nb, ops = model_ops()
    up, dn, pr = qo.combine_terms(ops, PARAMS, ns)
    _, nup, ndn = sector_of(NX, NY)
    S = qo.Sector(ns, nup, ndn, up, dn, pr)
    x = np.random.default_rng(1).standard_normal(S.dim)
    x /= np.linalg.norm(x)
    y = np.zeros(S.dim)
    S.mult_add(x, y, nthreads=threads)  # warm-up (page faults)
    t0 = time.perf_counter()
    for _ in range(steps):
        S.mult_add(x, y, nthreads=threads)
    dt = (time.perf_counter() - t0) / steps
    return BYTES_PER_STATE * S.dim / dt / 1e9, dt


def port_calibration():
    """The port's serial product against the reference's own serial
    Hamiltonian_Factorized::mult_add on the same 4x4 sector and host
    (oracle/calibrate_port.py; the reference's product is single-threaded),
    or None when that record is absent."""
    path = os.path.join(ROOT, "oracle", "port_calibration.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        c = json.load(f)
    return {"port_over_reference_serial_speed": c["port_over_reference_speed"],
            "reference_serial_s": c["reference_mult_add_s"],
            "port_serial_s": c["port_mult_add_1thread_s"], "host": c["host"],
            "note": "the reference's product runs on one thread"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # a bounded sample: each CPU product takes ~0.5 s on 16 Arm cores, so at
    # most 20 of them are timed whatever --steps asks of the device arm
    steps = max(1, min(args.steps, 20))
    gbs, dt = cpu_port_timing(steps, threads)
    sample = f"{steps} full products y += H x on the 4x4 N=16 Sz=0 sector, {threads} threads"
    line = {"impl": "reference", "metric": METRIC, "value": gbs, "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample, "calibration": port_calibration()},
            "e2e": {"value": gbs, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_gpu(args):
    import torch
    import pyqcm_gb300 as pg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pg._lib.check(pg.lib().qcmg_set_device(local))
    ns, nb, ops = model_ops()
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, PARAMS, sector_of(NX, NY)[0])
    D = H.dim
    # a dedicated stream: torch's legacy default stream has handle 0, which
    # the engine would read as "use your own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    H.set_stream(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
    x /= torch.linalg.vector_norm(x)
    fast = H.fx_available()
    if fast:
        # Krylov vectors of the fast path are device-resident fixed point
        qx = torch.empty(D, dtype=torch.int64, device="cuda")
        qy = torch.empty(D, dtype=torch.int64, device="cuda")
        E, mb = pg._lib.c_int(), pg._lib.c_int()
        pg._lib.check(pg.lib().qcmg_fx_from_f64(D, x.data_ptr(), qx.data_ptr(), E, mb,
                                                stream.cuda_stream))
        qy.copy_(qx)
        ey = [E.value]

        def step():  # y <- y + H x
            ey[0] = H.matvec_fx_device(qx.data_ptr(), E.value, mb.value, qy.data_ptr(),
                                       asynchronous=True, Ey_in=ey[0])
        y = qy
        kernels = ["k_fx_passU4", "k_fx_passD5"]
    else:
        y = x.clone()
        step = lambda: H.matvec_device(x.data_ptr(), y.data_ptr(), asynchronous=True, accumulate=True)
        kernels = ["k_matvec_f64"]
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        t_all0.record(stream)
        for k in range(args.steps):
            starts[k].record(stream)
            step()
            ends[k].record(stream)
        t_all1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    y_sum = float(torch.sum(torch.abs(y.double())).item())  # surfaces any asynchronous fault
    if not (y_sum > 0.0):
        raise RuntimeError("product produced an empty result")
    total_ms = t_all0.elapsed_time(t_all1)
    per_launch = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    bytes_step = BYTES_PER_STATE * D
    value = bytes_step * args.steps * world / (total_ms * 1e-3) / 1e9
    avg_launch_ms = sum(per_launch) / len(per_launch)
    achieved = bytes_step / (avg_launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()

    # The FP64 product (k_matvec_f64, any hop values) on the same sector and
    # vectors: the arithmetic the reference's mult_add performs, timed the
    # same way; the fixed-point line above is the fast path of this product.
    fp64 = None
    if fast and not args.no_fp64:
        yf = x.clone()
        H.set_path(False)
        stepf = lambda: H.matvec_device(x.data_ptr(), yf.data_ptr(), asynchronous=True,
                                        accumulate=True)
        for _ in range(max(args.warmup, 3)):
            stepf()
        nf = max(3, min(args.steps, 10))
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(nf):
            stepf()
        f1.record(stream)
        torch.cuda.synchronize()
        H.set_path(True)
        ms_f = f0.elapsed_time(f1) / nf
        gbs_f = bytes_step / (ms_f * 1e-3) / 1e9
        fp64 = {"value": gbs_f, "unit": UNIT, "ms_per_step": ms_f, "steps": nf,
                "frac": gbs_f / peak, "kernels": ["k_matvec_f64"], "dtype": "f64"}
        del yf

    # e2e through the public host API (Hamiltonian.mult_add, the reference's
    # mult_add): pinned host x and y in, y out, every step.
    xh = torch.empty(D, dtype=torch.float64, pin_memory=True)
    xh.copy_(x.cpu())
    xn = xh.numpy()
    yh = torch.zeros(D, dtype=torch.float64, pin_memory=True)
    yn = yh.numpy()
    e2e_steps = max(3, min(args.steps, 10))
    H.set_stream(0)
    for _ in range(max(args.warmup, 3)):  # warm-up: buffers, copy stream, first-touch costs
        H.mult_add(xn, yn)
    e2e_t = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        H.mult_add(xn, yn)
        e2e_t.append(time.perf_counter())
    e2e_s = (e2e_t[-1] - t0) / e2e_steps
    e2e_val = bytes_step * world / e2e_s / 1e9
    e2e_each = [1e3 * (b - a) for a, b in zip([t0] + e2e_t[:-1], e2e_t)]
    e2e_ms = sorted(e2e_each)
    del yh, yn

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64" if fast else "f64",
            "data": "synthetic", "config": workload_config(D),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": UNIT,
                         "frac": achieved / peak, "traffic": profile_traffic(),
                         "peak_kind": peak_kind, "kernels": kernels},
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 16 * D,
                    "d2h_bytes_per_step": 8 * D, "steps": e2e_steps,
                    "step_ms": {"min": e2e_ms[0], "median": e2e_ms[len(e2e_ms) // 2],
                                "max": e2e_ms[-1], "each": [round(v, 3) for v in e2e_each]}},
            "gpu_launches": args.steps * len(kernels)}
    if fp64:
        line["fp64_product"] = fp64
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        gbs, dt = cpu_port_timing(1, threads)
        line["cpu_baseline"] = {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"1 full product y += H x on the same sector, "
                                          f"{threads} threads ({dt:.2f} s)",
                                "calibration": port_calibration()}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def _fp64_peak():
    """FP64 FMA rate of this device in TFLOP/s, measured now by the
    library's probe (qcmg_fp64_fma_rate: eight FMA chains per thread, 8
    blocks of 256 threads per SM)."""
    from pyqcm_gb300 import _lib
    r = _lib.c_double()
    _lib.check(_lib.lib().qcmg_fp64_fma_rate(_lib.ctypes.byref(r)))
    return r.value


def run_lanczos(args):
    """4x4 N=16 Lanczos ground state to 1e-10.  Default: the reference's
    recurrence (no reorthogonalization), energy only, on the fixed-point
    path: time to solution and the per-iteration bytes (product 24 D + fused
    update/norm 16 D).  --reorth R: full reorthogonalization (classical
    Gram-Schmidt twice per step) against at most R vectors held in HBM, with
    an explicit restart from the Ritz vector at the cap; the products and
    the Gram-Schmidt sweeps are timed apart on the device."""
    import numpy as np
    import torch
    import pyqcm_gb300 as pg
    torch.cuda.set_device(0)
    ns, nb, ops = model_ops()
    m = pg.ClusterModel(ns, nb)
    for name, (typ, els) in ops.items():
        m.new_operator(name, typ, els)
    H = pg.Hamiltonian(m, PARAMS, sector_of(NX, NY)[0])
    D = H.dim
    peak, kind = measured_peak()
    ref = None
    gpath = os.path.join(ROOT, "tests", "golden", "large_4x4.npz")
    if (NX, NY, NEL) == (4, 4, None) and os.path.exists(gpath):
        ref = float(np.load(gpath)["lz_E0"])  # the reference's LanczosEigenvalue
    cfg = {"workload": f"{NX}x{NY} Hubbard cluster, t=1 U=8 mu=4, sector "
                       f"{sector_of(NX, NY)[0]} (dim {D:,}), Lanczos to 1e-10", "dim": D}
    if args.reorth:
        H.lanczos(tol=1e-10, max_iter=1000, reorth=args.reorth, want_psi=False)  # warm-up
        t0 = time.perf_counter()
        e0, _, alpha, _ = H.lanczos(tol=1e-10, max_iter=1000, reorth=args.reorth, want_psi=False)
        dt = time.perf_counter() - t0
        st = H.lanczos_stats()
        prod = st["product_ms"] * 1e-3
        cfg["workload"] += f", full reorthogonalization (at most {args.reorth} vectors in HBM)"
        cfg["reorth_vectors"] = args.reorth
        rgbs = st["reorth_bytes"] / (st["reorth_ms"] * 1e-3) / 1e9
        print(json.dumps({
            "metric": "lanczos_reorth_ground_state_s", "value": dt, "unit": "s",
            "higher_is_better": False, "E0": e0, "E0_reference": ref,
            "E0_rel_diff": None if ref is None else abs(e0 - ref) / abs(ref),
            "restarts": st["restarts"], "vectors_held": st["vectors"],
            "last_cycle_iterations": st["cycle"],
            "product_s": prod, "reorth_s": st["reorth_ms"] * 1e-3,
            "reorth_bytes": st["reorth_bytes"], "reorth_gbs": rgbs,
            "reorth_roofline": {"bound": "hbm", "achieved": rgbs, "peak": peak, "unit": "GB/s",
                                "frac": rgbs / peak, "peak_kind": kind,
                                "kernels": ["k_multidot", "k_multiaxpy"]},
            "dtype": "f64 (vectors, Gram-Schmidt); int64 (product)", "data": "synthetic",
            "config": cfg}))
        return
    e0, _, alpha, _ = H.lanczos(tol=1e-10, max_iter=600, want_psi=False)  # warm-up run
    t0 = time.perf_counter()
    e0, _, alpha, _ = H.lanczos(tol=1e-10, max_iter=600, want_psi=False)
    dt = time.perf_counter() - t0
    nit = len(alpha)
    per_iter = dt / nit
    gbs = 40.0 * D / per_iter / 1e9
    print(json.dumps({"metric": "lanczos_ground_state_s", "value": dt, "unit": "s",
                      "higher_is_better": False, "iterations": nit, "E0": e0,
                      "E0_reference": ref,
                      "E0_rel_diff": None if ref is None else abs(e0 - ref) / abs(ref),
                      "ms_per_iteration": per_iter * 1e3,
                      "bytes_per_iteration": 40 * D, "gbs_per_iteration": gbs,
                      "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                   "frac": gbs / peak, "peak_kind": kind},
                      "dtype": "int64", "data": "synthetic", "config": cfg}))


def _vca_3x4():
    """3x4 cluster, t=1 t'=-0.3 U=8 mu=4, AF Weiss field M (the VCA case)."""
    import pyqcm_gb300 as pg
    from pyqcm_gb300.lattice import LatticeModel
    cm = pg.ClusterModel(12, 0)
    sites = [(x, y, 0) for y in range(3) for x in range(4)]
    # superlattice (4,0), (1,3): the Neel wavevector is commensurate with it
    lm = LatticeModel(cm, sites, [(4, 0, 0), (1, 3, 0)])
    lm.interaction_operator("U", 1.0)
    lm.hopping_operator("t", (1, 0, 0), -1.0)
    lm.hopping_operator("t", (0, 1, 0), -1.0)
    lm.hopping_operator("tp", (1, 1, 0), -1.0)
    lm.hopping_operator("tp", (-1, 1, 0), -1.0)
    lm.density_wave("M", "Z", (1, 1, 0), 1.0, 0.0)
    lm.set_target_sectors("R0:N12:S0")
    lm.set_parameters({"t": 1.0, "tp": -0.3, "U": 8.0, "mu": 4.0, "M": 0.0, "M_1": 0.1})
    return lm


def _lattice_oracle():
    """The CPU oracle of the lattice layer (the CPU-baseline legs only)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lattice_oracle
    import qcm_oracle
    qcm_oracle.build()
    return lattice_oracle


def _cpu_cluster(lm, spins, threads):
    """The oracle's cluster solve of a lattice model's cluster: (lattice
    oracle module, E0, {spin_down: (e, v)}, {spin_down: (tc, tcb, eb)})."""
    lo = _lattice_oracle()
    lm.finalize()
    cm, vals = lm.cluster, lm.cluster_values()
    e0, Q = lo.cluster_lehmann(cm.operators, vals, cm.n_orb, cm.n_sites, lm.target_sectors, spins,
                               threads)
    blocks = {sd: lo.one_body_blocks(cm.operators, vals, cm.n_orb, cm.n_sites, sd) for sd in spins}
    return lo, e0, Q, blocks


def cpu_sef_baseline(w, wt, threads, sample=32):
    """The VCA Potthoff functional of the 3x4 case on the CPU oracle: the
    cluster solve in full (Lanczos, band-Lanczos Q-matrices of both spins),
    the 128x128 k grid integral on `sample` of the frequencies, scaled to
    all of them."""
    import numpy as np
    lm = _vca_3x4()
    t0 = time.perf_counter()
    lo, _, Q, blocks = _cpu_cluster(lm, (False, True), threads)
    t_solve = time.perf_counter() - t0
    idx = np.unique(np.linspace(0, len(w) - 1, sample).round().astype(int))
    t1 = time.perf_counter()
    for sd in (False, True):
        R, els, hdiff, _ = lm.fourier(sd)
        _, tcb, eb = blocks[sd]
        B, ldg = lo.base([(Q[sd][0], Q[sd][1], 1.0)], tcb, eb, hdiff, 1j * w[idx])
        lo.sef_grid(B, ldg, wt[idx], R, els, (128, 128, 1), threads)
    t_grid = (time.perf_counter() - t1) * len(w) / len(idx)
    return {"value": t_solve + t_grid, "unit": "s", "cores": threads, "kind": "port",
            "cluster_solve_s": t_solve, "grid_s": t_grid,
            "sample": f"the cluster solve in full; the 128x128 k integral of both spins on "
                      f"{len(idx)} of the {len(w)} frequencies, scaled to all"}


def run_sef(args):
    """VCA Potthoff functional on the 128x128 k grid x 256 Gauss-Legendre
    frequencies (2 spins, 12x12 blocks): the cluster solve (ground state +
    Green function, FP64 product since t' != t) and the grid integral."""
    import torch
    from pyqcm_gb300 import _lib, lattice as lat
    torch.cuda.set_device(0)
    lat.set_wavevector_grid(128, 128, 1)
    w, wt = lat.legendre_frequency_grid(1.0, 10.0, 64, 128, 64)
    lat.discrete_integration_grid(w, wt)
    lm = _vca_3x4()
    inst = lm.instance()
    t0 = time.perf_counter()
    omega = inst.Potthoff_functional()
    t_total = time.perf_counter() - t0
    blocks = inst._spin_blocks()
    t1 = time.perf_counter()
    for blk in blocks.values():
        out = _lib.c_double()
        _lib.check(_lib.lib().qcmg_sef_grid(blk._h, len(w), _lib.ptr(w), _lib.ptr(wt), 128, 128, 1,
                                            out))
    t_grid = time.perf_counter() - t1
    L = 12
    points = 128 * 128 * len(w) * len(blocks)
    flops = points * (8 * L ** 3 + 8 * L ** 3 / 3)  # per-point count of the reference's integrand
    lu = points * 8 * L ** 3 / 3  # executed FP64 flops of one complex LU per point
    peak = _fp64_peak()
    line = {"metric": "vca_sef_s_per_M_value", "value": t_total, "unit": "s",
            "higher_is_better": False, "omega": omega, "sef_grid_s": t_grid,
            "points": points, "points_per_s": points / t_grid,
            "alg_tflops": flops / t_grid / 1e12,
            "lu_tflops": lu / t_grid / 1e12, "fp64_peak_tflops": peak,
            "lu_frac_of_fp64": lu / t_grid / 1e12 / peak,
            "fp64_peak_kind": "measured now (qcmg_fp64_fma_rate)",
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "3x4 cluster t=1 t'=-0.3 U=8 mu=4 M_1=0.1, sector "
                                   "R0:N12:S0, 128x128 k x 256 frequencies, 2 spins"}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sef_baseline(w, wt, os.cpu_count() or 1)
    print(json.dumps(line))


def run_cpt(args):
    """CPT spectral function of the 8-site chain: 256 k x 512 real
    frequencies in [-8, 8], eta = 0.1."""
    import numpy as np
    import torch
    import pyqcm_gb300 as pg
    from pyqcm_gb300.lattice import LatticeModel
    torch.cuda.set_device(0)
    cm = pg.ClusterModel(8, 0)
    lm = LatticeModel(cm, [(i, 0, 0) for i in range(8)], [(8, 0, 0)])
    lm.interaction_operator("U", 1.0)
    lm.hopping_operator("t", (1, 0, 0), -1.0)
    lm.set_target_sectors("R0:N8:S0")
    lm.set_parameters({"t": 1.0, "U": 4.0, "mu": 2.0})
    inst = lm.instance()
    k = np.zeros((256, 3))
    k[:, 0] = np.arange(256) / 256.0
    w = np.linspace(-8.0, 8.0, 512)
    t0 = time.perf_counter()
    A = inst.spectral_function(w, k, eta=0.1)  # includes the cluster solve
    t_first = time.perf_counter() - t0
    times = []
    for _ in range(max(args.steps, 3)):  # median of repeated maps
        t1 = time.perf_counter()
        A = inst.spectral_function(w, k, eta=0.1)
        times.append(time.perf_counter() - t1)
    t_map = float(np.median(times))
    line = {"metric": "cpt_spectral_map_s", "value": t_map, "unit": "s",
            "higher_is_better": False, "with_cluster_solve_s": t_first,
            "repeats": len(times), "min_s": min(times),
            "points": int(A.size), "points_per_s": A.size / t_map,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "8-site chain t=1 U=4 mu=2, 256 k x 512 w in [-8,8], "
                                   "eta=0.1"}}
    if not args.no_cpu_baseline:
        # the same map on the CPU oracle (cluster solve timed apart, as the
        # repeated maps above reuse the solved cluster)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        lo, _, Q, blocks = _cpu_cluster(lm, (False,), threads)
        t_solve = time.perf_counter() - t0
        R, els, hdiff, gpos = lm.fourier(False)
        _, tcb, eb = blocks[False]
        t1 = time.perf_counter()
        B, _ = lo.base([(Q[False][0], Q[False][1], 1.0)], tcb, eb, hdiff, w + 0.1j)
        g = lo.cpt(B, R, els, k @ lm.S.T, gpos, threads)
        t_cpu = time.perf_counter() - t1
        line["cpu_baseline"] = {"value": t_cpu, "unit": "s", "cores": threads, "kind": "port",
                                "cluster_solve_s": t_solve,
                                "max_abs_diff": float(np.max(np.abs(-g.imag - A))),
                                "sample": "the whole map (256 k x 512 w)"}
    print(json.dumps(line))


def cdmft_instances(n, n_bath, seed=0, n_hyb=None):
    """Seeded CDMFT instances of the batched-CDMFT config: U ~ U[0,12],
    mu ~ U[0,U], bath energies ~ U[-3,3], hybridizations ~ U[0,1] (t = 1,
    t' = 0); n_hyb hybridizations (default one per bath orbital)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        U = rng.uniform(0, 12)
        mu = rng.uniform(0, U)
        eb = rng.uniform(-3, 3, n_bath)
        tb = rng.uniform(0, 1, n_hyb or n_bath)
        out.append((U, mu, eb, tb))
    return out


def cpu_cdmft_baseline(nb, hyb, sector, names, seed, mean_iterations, threads):
    """One CDMFT iteration of the first instance on the CPU oracle: the
    impurity ground state and band-Lanczos Q-matrix, the host function on the
    64x64 k grid x 200 Matsubara frequencies, the SciPy trf bath fit; points
    per hour at the GPU run's mean iterations per point."""
    import numpy as np
    from pyqcm_gb300.cdmft import plaquette_bath_model
    U, mu, eb, tb = cdmft_instances(1, nb, seed=seed, n_hyb=hyb * nb)[0]
    lm = plaquette_bath_model(nb, sector, hybridizations=hyb)
    params = {"t": 1.0, "tp": 0.0, "U": U, "mu": mu}
    params.update({n: float(v) for n, v in zip(names, np.concatenate([eb, tb]))})
    lm.set_parameters(params)
    wn = np.array([(2 * n + 1) * np.pi / 50.0 for n in range(200)])
    t0 = time.perf_counter()
    lo, _, Q, blocks = _cpu_cluster(lm, (False,), threads)
    t_solve = time.perf_counter() - t0
    R, els, hdiff, _ = lm.fourier(False)
    _, tcb, ebd = blocks[False]
    host = lo.cdmft_host([(Q[False][0], Q[False][1], 1.0)], tcb, ebd, hdiff, R, els, wn, 64,
                         lm.dim, threads)
    t_host = time.perf_counter() - t0 - t_solve
    cm, vals = lm.cluster, lm.cluster_values()
    cnames = [n[:-2] for n in names]
    lo.bath_fit(cm.operators, vals, cnames, cm.n_orb, cm.n_sites, host, wn, np.ones(len(wn)),
                [vals[n] for n in cnames])
    t_iter = time.perf_counter() - t0
    return {"value": 3600.0 / (t_iter * mean_iterations), "unit": "points/h", "cores": threads,
            "kind": "port", "s_per_iteration": t_iter, "impurity_s": t_solve, "host_s": t_host,
            "fit_s": t_iter - t_solve - t_host,
            "sample": f"one CDMFT iteration of instance 0 (impurity solve, host function, bath "
                      f"fit), scaled by the GPU run's {mean_iterations:.2f} mean iterations per "
                      f"point"}


def run_cdmft(args):
    """CDMFT loops of the plaquette + bath model to convergence, `--concurrency`
    loops in flight at a time on the device (host threads, one loop each):
    converged points per hour.  8 baths: 8 energies + 16 hybridizations (two
    per bath orbital), the batched-CDMFT configuration; 4 baths: one each."""
    import numpy as np
    import torch
    from pyqcm_gb300.cdmft import CDMFT, bath_names, plaquette_bath_model, run_batched, run_many
    torch.cuda.set_device(0)
    nb = args.bath or 8
    hyb = 2 if nb == 8 else 1
    sector = {4: "R0:N8:S0", 8: "R0:N12:S0"}[nb]
    names = bath_names(nb, hyb)
    loops = []
    for U, mu, eb, tb in cdmft_instances(args.samples or 32, nb, seed=args.seed, n_hyb=hyb * nb):
        lm = plaquette_bath_model(nb, sector, hybridizations=hyb)
        params = {"t": 1.0, "tp": 0.0, "U": U, "mu": mu}
        params.update({n: float(v) for n, v in zip(names, np.concatenate([eb, tb]))})
        lm.set_parameters(params)
        loops.append(CDMFT(lm, names, grid=(399 * np.pi / 50, 50.0), kside=64, maxiter=64,
                           fit=args.fit))
    t_all = time.perf_counter()
    if args.batched:
        res = run_batched(loops, workers=args.concurrency, chunk=args.chunk, groups=args.groups)
    else:
        res = run_many(loops, workers=args.concurrency)
    total = time.perf_counter() - t_all
    rows = []
    for c, (x, secs, err) in zip(loops, res):
        why = "" if err is None else f"{type(err).__name__}: {err}"[:160]
        rows.append((err is None, max(c.niter, len(c.history)), secs, c.time_ed, c.time_fit,
                     c.dist, why))
    conv = [r for r in rows if r[0]]
    failures = sorted({r[6] for r in rows if not r[0]})
    line = {
        "metric": "cdmft_converged_points_per_hour", "value": len(conv) / total * 3600.0,
        "unit": "points/h", "higher_is_better": True, "samples": len(rows),
        "converged": len(conv), "mean_iterations": float(np.mean([r[1] for r in rows])),
        "s_per_point": total / max(len(rows), 1),
        "s_per_iteration": sum(r[2] for r in rows) / max(sum(r[1] for r in rows), 1),
        "concurrency": args.concurrency, "bath_fit": args.fit,
        "driver": f"run_batched (lockstep in {args.groups} group(s): batched ground states and "
                  "bath fits)" if args.batched
        else "run_many (independent loops in host threads)",
        "impurity_and_host_s": sum(r[3] for r in rows), "bath_fit_s": sum(r[4] for r in rows),
        "failures": failures, "iteration": "broyden",
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"2x2 plaquette + {nb} bath orbitals ({nb} energies, {hyb * nb} "
                               f"hybridizations), sector {sector}, 200 Matsubara frequencies "
                               f"(beta=50), 64x64 k grid, Broyden CDMFT to the parameters test (1e-4)",
                   "instances": "seeded U~U[0,12], mu~U[0,U], eb~U[-3,3], tb~U[0,1]"}}
    if not args.no_cpu_baseline:
        mean_it = float(np.mean([r[1] for r in rows]))
        line["cpu_baseline"] = cpu_cdmft_baseline(nb, hyb, sector, names, args.seed, mean_it,
                                                  os.cpu_count() or 1)
    print(json.dumps(line))


def run_lanczos_batch(args):
    """Ground states of many uneven impurity sectors: `--samples` seeded
    instances of the 2x2 plaquette + 4 bath orbitals (U ~ U[0,12],
    mu ~ U[0,U], eb ~ U[-3,3], tb ~ U[0,1]), each in its sectors N = 7, 8, 9
    (3,920, 4,900 and 3,920 states), solved by Lanczos to 1e-12: all sectors
    at once (qcmg_lanczos_batch: each sector's steps replayed from a captured
    CUDA graph, all sectors side by side) against one sector at a time
    through the host-driven recurrence (the same FP64 arithmetic); sector
    solves per second both ways, and the energies must agree bit for bit."""
    import numpy as np
    import torch
    import pyqcm_gb300 as pg
    from pyqcm_gb300.cdmft import bath_names, plaquette_bath_model
    torch.cuda.set_device(0)
    nb = args.bath or 4
    hyb = 2 if nb == 8 else 1
    names = [n[:-2] for n in bath_names(nb, hyb)]
    no = 4 + nb
    if args.all_sectors:  # every (N_up, N_dn) with N_up >= N_dn: dims 1 to C(no, no/2)^2
        sectors = [f"R0:N{u + d}:S{u - d}" for u in range(no + 1) for d in range(u + 1)]
    else:
        sectors = ["R0:N7:S1", "R0:N8:S0", "R0:N9:S1"]
    hs = []
    for U, mu, eb, tb in cdmft_instances(args.samples or (16 if args.all_sectors else 256), nb,
                                         seed=args.seed, n_hyb=hyb * nb):
        lm = plaquette_bath_model(nb, "R0:N8:S0", hybridizations=hyb)
        lm.finalize()
        vals = {"t": 1.0, "U": U, "mu": mu}
        vals.update({n: float(v) for n, v in zip(names, np.concatenate([eb, tb]))})
        for sec in sectors:
            h = pg.Hamiltonian(lm.cluster, vals, sec)
            h.set_path(False)
            hs.append(h)
    pg.lanczos_batch(hs[:8], tol=1e-12, chunk=args.chunk, raise_errors=False)  # warm-up
    t0 = time.perf_counter()
    res = pg.lanczos_batch(hs, tol=1e-12, chunk=args.chunk, raise_errors=False)
    t_batch = time.perf_counter() - t0
    for h in hs[:8]:
        try:
            h.lanczos(tol=1e-12, want_psi=False)
        except pg.QcmgError:
            pass

    def one(h):
        try:
            return h.lanczos(tol=1e-12, want_psi=False)[0]
        except pg.QcmgError:  # the same sectors fail in both runs (the limit of the recurrence)
            return None
    t1 = time.perf_counter()
    single = [one(h) for h in hs]
    t_single = time.perf_counter() - t1
    ok = [k for k, r in enumerate(res) if r[3] is None]
    same = all(res[k][0] == single[k] for k in ok) and all(
        (single[k] is None) == (res[k][3] is not None) for k in range(len(hs)))
    iters = [res[k][2] for k in ok]
    print(json.dumps({
        "metric": "lanczos_batch_sector_solves_per_s", "value": len(hs) / t_batch,
        "unit": "solves/s", "higher_is_better": True, "sectors": len(hs),
        "batched_s": t_batch, "one_at_a_time_s": t_single,
        "one_at_a_time_solves_per_s": len(hs) / t_single, "speedup": t_single / t_batch,
        "mean_iterations": float(np.mean(iters)), "min_iterations": int(min(iters)),
        "max_iterations": int(max(iters)), "chunk": args.chunk, "bitwise_equal": same,
        "not_converged": len(hs) - len(ok),
        "dtype": "f64", "data": "synthetic",
        "dims": [int(min(h.dim for h in hs)), int(max(h.dim for h in hs))],
        "states": int(sum(h.dim for h in hs)),
        "config": {"workload": f"{len(hs) // len(sectors)} seeded 2x2 plaquette + {nb} bath "
                               f"instances x " + (f"all {len(sectors)} sectors N_up >= N_dn"
                                                  if args.all_sectors else
                                                  "sectors N=7,8,9 (3,920 / 4,900 / 3,920 states)")
                               + ", Lanczos to 1e-12",
                   "instances": "U~U[0,12], mu~U[0,U], eb~U[-3,3], tb~U[0,1]"}}))


def run_warmstart(args):
    """The learned warm start: train the device MLP on converged CDMFT solves,
    then run CDMFT on held-out points from the default bath and from the
    network's prediction, all loops of a run at once (lockstep driver), to
    the parameters test --accur; wall time and iterations of both, and the
    largest difference between the two runs' converged baths."""
    import numpy as np
    import torch
    from pyqcm_gb300 import warmstart as ws
    torch.cuda.set_device(0)
    nb = args.bath or 8
    import glob
    paths = (args.warm_data.split(",") if args.warm_data else sorted(glob.glob(
        os.path.join(ROOT, "pyqcm_gb300", "data", f"warmstart_{nb}bath_train*.npz"))))
    sets = [ws.load(p) for p in paths]
    P, Y = np.concatenate([a for a, _ in sets]), np.concatenate([b for _, b in sets])
    t0 = time.perf_counter()
    m, loss = ws.train(P, Y, epochs=args.epochs)
    t_train = time.perf_counter() - t0
    Ptest = ws.sample_params(args.samples or 512, seed=args.seed + 1000)  # held out: another seed
    r = ws.evaluate_batched(m, Ptest, nb, accur=args.accur, groups=args.groups,
                            accur_bath=args.accur_bath, accur_dist=args.accur_bath * 1e-2)
    ip, iw = np.array(r["iters_plain"]), np.array(r["iters_warm"])
    print(json.dumps({
        "metric": "cdmft_warm_start_speedup", "value": r["s_plain"] / r["s_warm"], "unit": "x",
        "higher_is_better": True, "held_out": r["points"], "both_converged": r["both_converged"],
        "plain_failed": r["plain_failed"], "train_points": len(P), "train_loss": loss,
        "train_s": t_train, "s_plain": r["s_plain"], "s_warm": r["s_warm"],
        "mean_iterations_plain": float(ip.mean()), "mean_iterations_warm": float(iw.mean()),
        "iteration_ratio": float(ip.sum() / iw.sum()),
        "max_bath_difference": float(max(r["max_dx"])),
        "median_bath_difference": float(np.median(r["max_dx"])),
        "median_prediction_error": float(np.median(r["pred_err"])),
        "fallbacks": r["fallbacks"],
        "dtype": "bf16 weights, f32 accumulate (MLP); f64 (CDMFT)", "data": "synthetic",
        "config": {"workload": f"2x2 plaquette + {nb} baths ({nb} energies, "
                               f"{ws.n_hyb(nb) * nb} hybridizations), MLP 4-256-256-"
                               f"{Y.shape[1]}, U in [4,12], t' in [-0.4,0], mu in [0.35U,0.5U]",
                   "convergence": f"parameters test {args.accur:g} (Broyden), bath fits to "
                                  f"xtol {args.accur_bath:g} / ftol {args.accur_bath * 1e-2:g}, "
                                  f"lockstep driver in {args.groups} groups"}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="qcmg", choices=["qcmg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the FP64 product measured beside the fixed-point one")
    ap.add_argument("--cluster", default="4x4",
                    help="NXxNY Hubbard cluster at half filling (profiling of smaller cases)")
    ap.add_argument("--electrons", type=int, default=None,
                    help="electrons in the sector (default: half filling)")
    ap.add_argument("--workload", default="product",
                    choices=["product", "lanczos", "lanczos-batch", "sef", "cpt", "cdmft",
                             "warmstart"],
                    help="product (the headline line) or one of the secondary measurements")
    ap.add_argument("--bath", type=int, default=None, choices=[4, 8],
                    help="bath orbitals (default 8: 8 energies + 16 hybridizations)")
    ap.add_argument("--samples", type=int, default=None,
                    help="instances of the CDMFT workload (default 32) or held-out points of "
                         "the warm-start workload (default 512)")
    ap.add_argument("--seed", type=int, default=0, help="seed of the CDMFT instances")
    ap.add_argument("--chunk", type=int, default=16,
                    help="lanczos-batch: recurrence steps per captured graph")
    ap.add_argument("--groups", type=int, default=1,
                    help="cdmft --batched: lockstep groups driven from their own threads")
    ap.add_argument("--batched", action="store_true",
                    help="cdmft: run the loops in lockstep with batched ground states and fits")
    ap.add_argument("--fit", default="device", choices=["device", "host"],
                    help="CDMFT bath fit: on the device (qcmg_bath_fit) or SciPy on the host")
    ap.add_argument("--concurrency", type=int, default=8,
                    help="CDMFT loops in flight at a time (one host thread each)")
    ap.add_argument("--reorth", type=int, default=0,
                    help="lanczos workload: full reorthogonalization against at most this many "
                         "vectors held in HBM (0: the reference's recurrence)")
    ap.add_argument("--all-sectors", action="store_true",
                    help="lanczos-batch: every (N_up >= N_dn) sector of each instance")
    ap.add_argument("--warm-data", default=None,
                    help="training sets of the warm-start workload, comma-separated (default: "
                         "every pyqcm_gb300/data/warmstart_<bath>bath_train*.npz)")
    ap.add_argument("--epochs", type=int, default=20000, help="training epochs of the warm-start MLP")
    ap.add_argument("--accur", type=float, default=3e-8,
                    help="warmstart: parameters test of both CDMFT runs")
    ap.add_argument("--accur-bath", type=float, default=1e-10,
                    help="warmstart: xtol of every bath fit of both runs (ftol 1e-2 of it)")
    args = ap.parse_args()
    global NX, NY, NEL
    NX, NY = (int(v) for v in args.cluster.split("x"))
    NEL = args.electrons
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "lanczos":
        run_lanczos(args)
    elif args.workload == "lanczos-batch":
        run_lanczos_batch(args)
    elif args.workload == "sef":
        run_sef(args)
    elif args.workload == "cpt":
        run_cpt(args)
    elif args.workload == "cdmft":
        run_cdmft(args)
    elif args.workload == "warmstart":
        run_warmstart(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
