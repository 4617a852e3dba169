"""Benchmark: 30-qubit ComplexDP gate layer (Haar-random U on every qubit + CZ brick), GB/s.

One step = one layer on a 2^30-amplitude ComplexDP register (16 GiB, far larger than L2):
30 Haar-random 2x2 gates (QR of a seeded complex Gaussian, phase-fixed), CZ on the 15 even
pairs, then the 14 odd pairs. The metric is the layer's algorithmic bytes -- 2*N*16 per
1-qubit gate and N*16 per controlled gate, the reference's own accounting
(src/highperfkernels.cpp:370, :478) -- divided by the layer time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--qubits 30] [--math emulated|native]

--impl reference times the reference's CPU implementation of the same layer on the host
cores (the reference library built from its sources when present, else the C restatement
in oracle/), on a 28-qubit sample of the workload. Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
for _p in (REPO, REPO / "intel-qs_gb300", REPO / "tests"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "30q gate-layer HBM GB/s (ComplexDP, algorithmic bytes)"
UNIT = "GB/s"
FALLBACK_HBM_GBS = 6800.0


def host_mem_available() -> int:
    """Bytes of host memory this process may still take (MemAvailable, capped by a cgroup
    limit when one is set)."""
    avail = 0
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        return 0
    for path in ("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory/memory.limit_in_bytes"):
        try:
            with open(path) as f:
                lim = f.read().strip()
            with open(path.replace("memory.max", "memory.current").replace("limit_in_bytes", "usage_in_bytes")) as f:
                used = int(f.read().strip())
            if lim.isdigit():
                avail = min(avail, int(lim) - used)
        except OSError:
            continue
    return avail


def max_over_ranks(value: float, dist=None, device: str = "cuda") -> float:
    """The largest value over all ranks (the slowest replica's time); value itself when
    running alone."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gbs(world: int, bytes_per_rank: int, seconds: float) -> float:
    """Whole-job throughput: every replica moves bytes_per_rank in `seconds` (the max over
    ranks)."""
    return world * bytes_per_rank / seconds / 1e9


def layer_bytes(n: int, amp_bytes: int = 16) -> int:
    N = 1 << n
    num_cz = (n // 2) + ((n - 1) // 2)
    return n * 2 * N * amp_bytes + num_cz * N * amp_bytes


def haar_layers(n: int, count: int, seed: int) -> list:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        mats = []
        for _q in range(n):
            z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / np.sqrt(2.0)
            q, r = np.linalg.qr(z)
            d = np.diag(r)
            mats.append(np.ascontiguousarray(q * (d / np.abs(d))))
        out.append(mats)
    return out


def apply_layer(reg, mats, n: int, on_1q=None) -> None:
    """Public-API layer: Apply1QubitGate on every qubit, then the CZ bricks."""
    for q in range(n):
        if on_1q is not None:
            on_1q(0)
        reg.Apply1QubitGate(q, mats[q])
        if on_1q is not None:
            on_1q(1)
    for j in range(n // 2):
        reg.ApplyCPauliZ(2 * j, 2 * j + 1)
    for j in range((n - 1) // 2):
        reg.ApplyCPauliZ(2 * j + 1, 2 * j + 2)


def peak_hbm() -> tuple[float, str]:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        import tempfile
        self.path = Path(tempfile.gettempdir()) / f"iqsg_bench_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "0x1", "1"):
                    reasons.add(nm)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_layer_gbs(n: int, layers: int, seed: int, threads: int | None = None, use_ref: bool = False) -> dict:
    """The same layer on the host cores: the reference library (when built here) or the
    C restatement (oracle/) with all OpenMP threads."""
    import oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle.set_threads(threads)
    kind = "reference" if (use_ref and oracle.ref_available()) else "port"
    reg = (oracle.RefRegister if kind == "reference" else oracle.OracleRegister)(n, "base", 0)
    mats = haar_layers(n, layers, seed)
    t0 = time.perf_counter()
    for l in range(layers):
        apply_layer(reg, mats[l], n)
    dt = time.perf_counter() - t0
    return {"kind": kind, "seconds": dt, "gbs": layers * layer_bytes(n) / dt / 1e9,
            "cores": threads or oracle.get_threads()}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.cpu_qubits
    import oracle
    oracle.build(ref=None)
    threads = os.cpu_count() or 1
    times, kind = [], None
    for s in range(args.warmup + args.steps):
        r = cpu_layer_gbs(n, 1, seed=100 + s, threads=threads, use_ref=True)
        kind = r["kind"]
        if s >= args.warmup:
            times.append(r["seconds"])
    t = statistics.median(times)
    value = layer_bytes(n) / t / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Haar-random gates)",
            "config": {"workload": f"gate layer: Haar U on each of {n} qubits + CZ brick, ComplexDP",
                       "qubits": n, "sample": f"one {n}-qubit layer per step (the 30q layer shape at {n} qubits)"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"one {n}-qubit layer per step, {threads} OpenMP threads"},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def regular_graph(n: int, degree: int, seed: int) -> list:
    """Seeded random regular graph: configuration model, redrawn until simple."""
    rng = np.random.default_rng(seed)
    while True:
        stubs = rng.permutation(np.repeat(np.arange(n), degree))
        pairs = stubs.reshape(-1, 2)
        edges = {tuple(sorted((int(a), int(b)))) for a, b in pairs}
        if all(a != b for a, b in edges) and len(edges) == len(pairs):
            return sorted(edges)


def qaoa_section(n: int = 26, p: int = 8, stream=None) -> dict:
    """QAOA MaxCut on a 3-regular graph: adjoint gradient vs central finite differences on
    the GPU (same forward kernels; h = 1e-6), and vs finite differences through the plain
    per-gate public API (cost vector + one RX kernel per qubit), ComplexDP."""
    import iqs_gb300 as iqs
    import torch
    edges = regular_graph(n, 3, seed=3)
    rng = np.random.default_rng(4)
    gammas, betas = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    circ = iqs.QaoaMaxCut(n, edges, stream=stream, checkpoint=True)
    circ.energy_and_grad(gammas, betas)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e, dg, db = circ.energy_and_grad(gammas, betas)
    t_adj = time.perf_counter() - t0
    t0 = time.perf_counter()
    fdg, fdb = circ.finite_difference_grad(gammas, betas, h=1e-6)
    t_fd = time.perf_counter() - t0
    g, fd = np.concatenate([dg, db]), np.concatenate([fdg, fdb])
    rel = float(np.max(np.abs(g - fd)) / np.max(np.abs(fd)))
    # One energy through the plain per-gate API, then 2P of them for the plain FD figure.
    adj = np.zeros((n, n), dtype=np.int32)
    for u, v in edges:
        adj[u, v] = adj[v, u] = 1
    diag = iqs.QubitRegister(n, "base", 0, stream=stream)
    iqs.InitializeVectorAsMaxCutCostFunction(diag, adj.reshape(-1))
    psi = iqs.QubitRegister(n, "++++", 0, stream=stream)

    def plain_energy():
        psi.Initialize("++++", 0)
        for gm, bt in zip(gammas, betas):
            iqs.ImplementQaoaLayerBasedOnCostFunction(psi, diag, -gm)
            for q in range(n):
                psi.ApplyRotationX(q, 2 * bt)
        return len(edges) - 2 * iqs.GetExpectationValueFromCostFunction(psi, diag)

    e_plain = plain_energy()
    t0 = time.perf_counter()
    plain_energy()
    t_plain = (time.perf_counter() - t0) * 2 * 2 * p
    del circ, diag, psi
    return {"workload": f"QAOA MaxCut, random 3-regular graph on {n} vertices ({len(edges)} edges), p={p}, "
                        f"16 parameters U[0, pi), ComplexDP, native FP64, checkpointed adjoint (2p saved states)",
            "energy": e, "energy_plain_api": e_plain,
            "adjoint_s": round(t_adj, 4), "adjoint_grads_per_s": round(1 / t_adj, 3),
            "fd_same_kernels_s": round(t_fd, 3), "fd_same_kernels_grads_per_s": round(1 / t_fd, 4),
            "speedup_vs_fd_same_kernels": round(t_fd / t_adj, 2),
            "fd_plain_api_s": round(t_plain, 3), "speedup_vs_fd_plain_api": round(t_plain / t_adj, 2),
            "max_rel_diff_adjoint_vs_fd": rel}


def batched_instances(count: int = 4096, seed_shape: int = 5, seed_obs: int = 6) -> list:
    rng = np.random.default_rng(seed_shape)
    ns = rng.integers(12, 21, size=count)
    ls = rng.integers(4, 13, size=count)
    orng = np.random.default_rng(seed_obs)
    out = []
    for n, L in zip(ns, ls):
        terms = [(float(orng.standard_normal()), "".join(orng.choice(list("IXYZ"), size=int(n)))) for _ in range(8)]
        out.append((int(n), int(L), terms))
    return out


def batched_section(count: int = 4096, loop_sample: int = 64) -> dict:
    """Hardware-efficient ansatz batch (ComplexSP): energies + adjoint gradients of every
    instance in one persistent launch replayed as a CUDA graph, against a per-circuit loop
    through the public API (forward energies only, sampled and scaled), and the same batch in
    ComplexDP as the FP64 reference for the error."""
    import iqs_gb300 as iqs
    inst = batched_instances(count)
    b = iqs.BatchedAnsatz(inst, precision="SP")
    params = np.random.default_rng(7).uniform(0, 2 * np.pi, b.num_params)
    table = b.autotune(params, with_grad=True, trials=1)
    best_fg = best_f = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        e32, g32 = b.run(params, with_grad=True)
        best_fg = min(best_fg, time.perf_counter() - t0)
        t0 = time.perf_counter()
        b.run(params)
        best_f = min(best_f, time.perf_counter() - t0)
    # FP64 reference on a subset (ComplexDP, same kernel).
    sub = list(range(0, count, max(1, count // 256)))
    bd = iqs.BatchedAnsatz([inst[i] for i in sub], precision="DP")
    pd = np.concatenate([params[b.param_slices()[i]] for i in sub])
    e64, g64 = bd.run(pd, with_grad=True)
    g32s = np.concatenate([g32[b.param_slices()[i]] for i in sub])
    e_err = float(np.max(np.abs(e32[sub] - e64)))
    g_err = float(np.max(np.abs(g32s - g64)) / max(1.0, np.max(np.abs(g64))))
    del bd
    # Per-circuit loop through the public API, forward energy only.
    rng = np.random.default_rng(8)
    pick = rng.choice(count, size=min(loop_sample, count), replace=False)
    t0 = time.perf_counter()
    loop_e = []
    for i in pick:
        n, L, terms = inst[i]
        prm = params[b.param_slices()[i]]
        r = iqs.QubitRegister(n, "base", 0, precision="SP")
        r.TurnOnFusion()
        for l in range(L):
            for q in range(n):
                r.ApplyRotationZ(q, prm[2 * (l * n + q)])
                r.ApplyRotationY(q, prm[2 * (l * n + q) + 1])
            for q in range(n - 1):
                r.ApplyCPauliZ(q, q + 1)
        e = 0.0
        for c, st in terms:
            qs = [q for q, ch in enumerate(st) if ch != "I"]
            e += r.ExpectationValue(qs, [{"X": 1, "Y": 2, "Z": 3}[st[q]] for q in qs], c) if qs else c
        loop_e.append(e)
    t_loop = (time.perf_counter() - t0) * count / len(pick)
    loop_err = float(np.max(np.abs(np.asarray(loop_e) - e32[pick])))
    gates = sum(L * (2 * n + n - 1) for n, L, _ in inst)
    return {"workload": f"{count} hardware-efficient ansatz instances, n ~ U{{12..20}}, L ~ U{{4..12}}, "
                        f"RZ RY per qubit + CZ ladder per layer, 8 Pauli strings each, ComplexSP",
            "gates": gates, "parameters": int(b.num_params), "amplitudes": int(b.total_amplitudes),
            "launch": {"threads": b.launch[0], "ctas_per_sm": b.launch[1],
                       "autotune_s": [[t, c, round(x, 4)] for t, c, x in table]},
            "forward_and_grad_s": round(best_fg, 4), "forward_s": round(best_f, 4),
            "circuits_per_s_with_grad": round(count / best_fg, 1),
            "per_circuit_loop_forward_s": round(t_loop, 3), "per_circuit_loop_sample": len(pick),
            "speedup_forward_vs_loop": round(t_loop / best_f, 2),
            "max_abs_energy_err_sp_vs_dp": e_err, "max_rel_grad_err_sp_vs_dp": g_err,
            "max_abs_energy_diff_vs_loop": loop_err}


def plain_section(reps: int = 5) -> dict:
    """The 20-qubit, 780-gate circuit (20 layers of Haar U on every qubit + CNOT bricks) from
    |0...0>, gate by gate and fused, ComplexDP in native and emulated arithmetic: time per
    circuit and the error against the amplitudes the reference itself computed
    (tests/golden/golden.npz, case plain_gate_by_gate_20q); the 16 MiB state stays in L2, so
    this reports time, not an HBM fraction. The C restatement of the reference's loops runs
    the same circuit on the host cores for comparison."""
    import iqs_gb300 as iqs
    import oracle
    from circuits import replay
    z = np.load(REPO / "tests" / "golden" / "golden.npz")
    name = "plain_gate_by_gate_20q"
    ops = json.loads(str(z[f"{name}/ops"]))
    idx, want = z[f"{name}/final_idx"], z[f"{name}/final"]
    from circuits import QUERIES
    out = {"workload": "20 qubits, 20 layers of (Haar U on every qubit + CNOT bricks), 780 gates, ComplexDP",
           "gates": sum(1 for name, _ in ops if name not in QUERIES)}
    for math in ("native", "emulated"):
        for fusion in (False, True):
            reg = iqs.QubitRegister(20, "base", 0, math=math)
            best = float("inf")
            for _ in range(reps):
                reg.Initialize("base", 0)
                if fusion:
                    reg.TurnOnFusion()
                reg.synchronize()
                t0 = time.perf_counter()
                replay(reg, ops)
                reg.ApplyFusedGates()
                reg.synchronize()
                best = min(best, time.perf_counter() - t0)
            err = float(np.max(np.abs(reg.GetStateVector()[idx] - want)))
            out[f"{math}{'_fused' if fusion else ''}"] = {"ms": round(best * 1e3, 2), "max_abs_err_vs_reference": err}
    o = oracle.OracleRegister(20, "base", 0)
    t0 = time.perf_counter()
    replay(o, ops)
    out["cpu_restatement_ms"] = round((time.perf_counter() - t0) * 1e3, 1)
    out["cpu_threads"] = oracle.get_threads()
    return out


def gate_bytes(ops, n: int, amp_bytes: int) -> int:
    """Algorithmic bytes of a gate list: 2*N*s per 1-qubit gate, N*s per controlled or
    swap-type gate (src/highperfkernels.cpp:370, :478-479)."""
    N = 1 << n
    one = {"Apply1QubitGate", "ApplyHadamard"}
    return sum((2 if name in one else 1) * N * amp_bytes for name, _ in ops)


def qft_brick_section(n: int = 30, layers: int = 40) -> dict:
    """QFT + 40 Haar/CZ brick layers from a seeded basis state: ComplexDP gate by gate and in
    fused passes (emulated arithmetic), ComplexSP in fused passes; errors against the
    amplitudes the reference itself computed (tests/golden/qft_brick.npz), SP fidelity
    against DP."""
    import hashlib
    import torch
    import iqs_gb300 as iqs
    from circuits import loads, qft_brick, qft_brick_start, replay
    ops = qft_brick(n, layers)
    start = qft_brick_start(n)
    fix = REPO / "tests" / "golden" / "qft_brick.npz"
    ref = None
    if fix.exists():  # the stored circuit (a list generated on another machine can differ in the last bit)
        z = np.load(fix)
        if f"n{n}/ops" in z.files:
            meta = json.loads(str(z[f"n{n}/meta"]))
            text = str(z[f"n{n}/ops"])
            if meta["layers"] == layers and meta["ops_sha256"] == hashlib.sha256(text.encode()).hexdigest():
                ops, start = loads(text), meta["start"]
                ref = (z[f"n{n}/idx"], z[f"n{n}/amps"])
    out = {"workload": f"{n}-qubit QFT (examples/quantum_fourier_transform.cpp gate order) + {layers} layers of "
                       f"(Haar U on every qubit + CZ brick), from basis state {start}",
           "gates": len(ops)}

    def timed(reg, fusion):
        if fusion:
            reg.TurnOnFusion()
        reg.synchronize()
        t0 = time.perf_counter()
        replay(reg, ops)
        sweeps = reg.ApplyFusedGates() if fusion else len(ops)
        reg.synchronize()
        return time.perf_counter() - t0, sweeps

    def sample_err(reg):
        if ref is None:
            return None
        v = torch.as_tensor(reg, device="cuda")[torch.as_tensor(ref[0], device="cuda")].cpu().numpy()
        return float(np.max(np.abs(v.astype(np.complex128) - ref[1])))

    dp = iqs.QubitRegister(n, "base", start, precision="DP", math="emulated")
    t_dp, _ = timed(dp, False)
    dpf = iqs.QubitRegister(n, "base", start, precision="DP", math="emulated")
    t_dpf, sweeps_dpf = timed(dpf, True)
    dpf_runs = dpf.counters()["df_runs"]
    dpf_err = sample_err(dpf)
    dpf_diff = float((torch.as_tensor(dpf, device="cuda") - torch.as_tensor(dp, device="cuda")).abs().max())
    del dpf
    sp = iqs.QubitRegister(n, "base", start, precision="SP")
    t_sp, sweeps = timed(sp, True)
    sp.Initialize("base", start)
    t_sp, sweeps = timed(sp, True)  # second run: warm
    a, b = torch.as_tensor(dp, device="cuda"), torch.as_tensor(sp, device="cuda")
    mx, ov, na, nb = 0.0, 0j, 0.0, 0.0
    for s0 in range(0, a.numel(), 1 << 26):
        x, y = a[s0:s0 + (1 << 26)], b[s0:s0 + (1 << 26)].to(torch.complex128)
        mx = max(mx, float((x - y).abs().max()))
        ov += complex(torch.vdot(x, y))
        na += float(torch.vdot(x, x).real)
        nb += float(torch.vdot(y, y).real)
    out.update({
        "dp_gate_by_gate": {"s": round(t_dp, 3), "launches": len(ops),
                            "gbs_algorithmic": round(gate_bytes(ops, n, 16) / t_dp / 1e9, 1),
                            "max_abs_err_vs_reference_sample": sample_err(dp)},
        "dp_fused": {"s": round(t_dpf, 3), "passes": sweeps_dpf, "double_float_storage_runs": dpf_runs,
                     "gbs_algorithmic": round(gate_bytes(ops, n, 16) / t_dpf / 1e9, 1),
                     "max_abs_err_vs_reference_sample": dpf_err, "max_abs_diff_vs_dp_gate_by_gate": dpf_diff},
        "sp_fused": {"s": round(t_sp, 3), "passes": sweeps,
                     "gbs_algorithmic": round(gate_bytes(ops, n, 8) / t_sp / 1e9, 1),
                     "max_abs_err_vs_reference_sample": sample_err(sp),
                     "max_abs_diff_vs_dp": mx, "fidelity_vs_dp": abs(ov) ** 2 / (na * nb)},
        "reference_sample": None if ref is None else f"{ref[0].size} amplitudes from the reference (ComplexDP)",
    })
    del a, b, dp, sp
    torch.cuda.empty_cache()
    return out


def trotter_section(n: int = 32, steps: int = 100, n_dp: int = 33, steps_dp: int = 4, grad_steps: int = 10,
                    tile_qubits: int = 0) -> dict:
    """Open XXZ chain (31 bonds at n = 32, J ~ U[0.5, 1.5] seed 7, delta = 0.8, dt = 0.05) from
    the Neel state: 100 Strang steps in ComplexSP with the 31 bond correlators, then the
    energy sum_b <Z_b Z_{b+1}> and its gradient w.r.t. every J_b by the checkpointed adjoint;
    a few steps of the same chain at 33 qubits in ComplexDP (128 GiB) for the HBM roofline;
    parity of the same 100-step circuit at 20 qubits against the oracle. The gradient runs
    over the first `grad_steps` Strang steps (all of them with grad_steps = steps)."""
    import torch
    import oracle
    from iqs_gb300 import _lib
    from iqs_gb300.trotter import XXZChain, bond_gate, strang_layers
    J = np.random.default_rng(7).uniform(0.5, 1.5, n - 1)
    out = {"workload": f"open XXZ chain, {n} qubits ComplexSP, delta 0.8, dt 0.05, {steps} Strang steps "
                       f"(even half steps merged), Neel start; bond gate = RXX RYY RZZ as one 2-qubit gate"}
    vec = (1 << n) * 8
    free = torch.cuda.mem_get_info()[0]
    every = None
    for c in (10, 20, 25, 50):
        if (2 + len(range(c, steps, c))) * vec + (16 << 30) <= free:
            every = c
            break
    chain = XXZChain(n, J, steps=steps, precision="SP", checkpoint_every=None, tile_qubits=tile_qubits)
    gates = sum(len(b) for b, _ in chain.layers())
    chain.psi.synchronize()
    t0 = time.perf_counter()
    zz = chain.bond_zz()
    chain.psi.synchronize()
    t_fwd = time.perf_counter() - t0
    fwd_sweeps = chain.sweeps_forward
    chain.sweeps_forward = 0
    norm_after = float(chain.psi.ComputeNorm())
    del chain
    gchain = XXZChain(n, J, steps=grad_steps, precision="SP",
                      checkpoint_every=every if (every and grad_steps > every) else None, tile_qubits=tile_qubits)
    gchain.forward()
    gchain.psi.synchronize()
    t0 = time.perf_counter()
    e, grad = gchain.energy_and_grad()
    t_grad = time.perf_counter() - t0
    N = 1 << n
    out["sp"] = {"gates": gates, "forward_s": round(t_fwd, 3), "forward_passes": fwd_sweeps,
                 "forward_gbs_algorithmic": round(gates * 2 * N * 8 / t_fwd / 1e9, 1),
                 "forward_pass_gbs": round(fwd_sweeps * 2 * N * 8 / t_fwd / 1e9, 1),
                 "zz_first4": [round(float(x), 8) for x in zz[:4]], "zz_mean": float(np.mean(zz)),
                 "norm_after_forward": norm_after,
                 "gradient": {"strang_steps": grad_steps, "energy": e,
                              "grad_first4": [round(float(x), 8) for x in grad[:4]],
                              "grad_norm": float(np.linalg.norm(grad)),
                              "forward_and_grad_s": round(t_grad, 3), "adjoint_passes": gchain.sweeps_backward,
                              "adjoint_pass_gbs": round(gchain.sweeps_backward * 4 * N * 8 /
                                                        max(t_grad - t_fwd * grad_steps / steps, 1e-9) / 1e9, 1),
                              "checkpoint_every_steps": gchain.checkpoint_every, "checkpoints": len(gchain._ckpt)}}
    del gchain
    # 33-qubit ComplexDP forward, emulated arithmetic: roofline of the fused passes.
    Jd = np.random.default_rng(7).uniform(0.5, 1.5, n_dp - 1)
    if (1 << n_dp) * 16 + (8 << 30) <= torch.cuda.mem_get_info()[0]:
        ch = XXZChain(n_dp, Jd, steps=steps_dp, precision="DP", checkpoint_every=None)
        ch.psi.SetMath("emulated")
        ch.forward()
        ch.psi.synchronize()
        ch.sweeps_forward = 0
        t0 = time.perf_counter()
        ch.forward()
        ch.psi.synchronize()
        t = time.perf_counter() - t0
        gd = sum(len(b) for b, _ in ch.layers())
        out["dp33"] = {"qubits": n_dp, "steps": steps_dp, "gates": gd, "passes": ch.sweeps_forward, "s": round(t, 3),
                       "gbs_algorithmic": round(gd * 2 * (1 << n_dp) * 16 / t / 1e9, 1),
                       "pass_gbs": round(ch.sweeps_forward * 2 * (1 << n_dp) * 16 / t / 1e9, 1),
                       "math": "emulated"}
        del ch
    # parity: the same 100-step circuit at 20 qubits, SP and DP, against the oracle
    n20 = 20
    J20 = np.random.default_rng(7).uniform(0.5, 1.5, n20 - 1)
    o = oracle.OracleRegister(n20, "base", sum(1 << q for q in range(1, n20, 2)))
    for bonds, tau in strang_layers(n20, 0.05, steps):
        for b in bonds:
            o.Apply2QubitGate(b + 1, b, bond_gate(0.5 * tau * J20[b], 0.8))
    want = np.asarray([o.ExpectationValue([b, b + 1], [3, 3], 1.0) for b in range(n20 - 1)])
    ost = o.GetStateVector()
    par = {}
    for prec in ("DP", "SP"):
        c20 = XXZChain(n20, J20, steps=steps, precision=prec, checkpoint_every=None)
        z20 = c20.bond_zz()
        par[prec] = {"max_abs_zz_err": float(np.max(np.abs(z20 - want))),
                     "max_abs_amp_err": float(np.max(np.abs(c20.psi.GetStateVector() - ost)))}
    out["parity_20q_vs_oracle"] = par
    return out


def run_ours(args) -> None:
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    import iqs_gb300 as iqs

    n = args.qubits
    # A dedicated (non-default) stream: the register queues every kernel on it and the
    # CUDA events below are recorded on the same stream.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    reg = iqs.QubitRegister(n, "base", 0, math=args.math, stream=stream.cuda_stream)
    for q in range(n):  # a dense state: every amplitude nonzero
        reg.ApplyHadamard(q)
    tuned = None
    if args.width:
        reg.SetSweepWidth(args.width)
        reg.SetSweepPipeline(args.pipeline)
        if args.math == "emulated":
            reg.SetNativeShare(args.native_share)
    elif args.fusion:
        from iqs_gb300.autotune import tune_fusion
        tuned = tune_fusion(reg)  # untimed: picks the pass width and kernel for this register
    if args.fusion:
        reg.TurnOnFusion()
    total = args.warmup + args.steps
    mats = haar_layers(n, total, seed=1000 + rank)

    def step(s, on_1q=None):
        """One layer through the public API; with fusion on, the queued gates are applied
        in fused passes by ApplyFusedGates (the reference's own fusion entry points)."""
        apply_layer(reg, mats[s], n, on_1q=on_1q)
        return reg.ApplyFusedGates() if args.fusion else n + (n // 2) + ((n - 1) // 2)

    # Warm-up (untimed).
    for s in range(args.warmup):
        step(s)
    barrier()

    # Timed region: K layers on the register's stream. Without fusion, event pairs also
    # bracket each 1-qubit gate launch (the dominant kernel).
    kev = []

    def mark(which):
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        if which == 0:
            kev.append([e, None])
        else:
            kev[-1][1] = e

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sweeps = 0
    c0 = reg.counters()
    start.record(stream)
    for s in range(args.warmup, total):
        sweeps += step(s, on_1q=None if args.fusion else mark)
    end.record(stream)
    barrier()
    c1 = reg.counters()
    # Kernels launched: one per sweep, except in double-float storage runs, which launch a
    # range check and two kernels per sweep (the FP64-storage one returns at once).
    df_runs = c1["df_runs"] - c0["df_runs"]
    df_launches = c1["df_launches"] - c0["df_launches"]
    df_sweeps = (df_launches - df_runs) // 2
    launches = sweeps - df_sweeps + df_launches
    clk = clocks.stop()
    ms = max_over_ranks(start.elapsed_time(end), dist)
    ms_per_step = ms / args.steps
    value = job_gbs(world, layer_bytes(n), ms_per_step * 1e-3)

    # Dominant kernel. Fused: every sweep in the timed region is a full pass over the state
    # (2*N*16 bytes), so the average pass time is the region time / sweeps (which also
    # charges the range checks and the launches that return at once to the passes).
    # Unfused: the 1-qubit gate kernel, timed by its event pairs.
    if args.fusion:
        k_avg = ms / sweeps
        if args.math != "emulated":
            kname = "k_sweep_native<double> (fused pass)"
        elif df_runs:
            kname = "k_sweep_dfs (fused pass, emulated FP64, double-float pairs between passes)"
        else:
            kname = "k_sweep_df (fused pass, emulated FP64)"
    else:
        k_avg = statistics.mean(a.elapsed_time(b) for a, b in kev)
        kname = "k_1q_df (1-qubit gate, emulated FP64)" if args.math == "emulated" else "k_1q<double>"
    peak, peak_src = peak_hbm()
    achieved = 2 * (1 << n) * 16 / (k_avg * 1e-3) / 1e9
    # DRAM bytes per launch: given on the command line, else the ratio ncu measured for the
    # fused emulated pass on a 27-qubit state (4.234 GB read + written per 4.295 GB pass; the
    # capture is too large to repeat at 30 qubits), scaled by the amplitudes of this pass.
    width_used = args.width or (tuned and tuned["width"])
    if args.traffic is not None:
        traffic, traffic_src = args.traffic, "command line"
    elif args.fusion and args.math == "emulated" and df_runs and width_used == 2:
        # ncu on k_sweep_dfs<2, pairs in, pairs out> at 27 qubits: 4.234 GB per 4.295 GB pass.
        traffic = round(4.234e9 / 4.295e9 * 2 * (1 << n) * 16)
        traffic_src = "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_sweep_dfs<2,1,1> at 27 qubits, scaled"
    elif args.fusion and args.math == "emulated" and not df_runs and width_used == 2:
        traffic = round(4.234e9 / 4.295e9 * 2 * (1 << n) * 16)
        traffic_src = "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_sweep_df<2> at 27 qubits, scaled"
    else:
        traffic, traffic_src = None, None

    # End to end through the public API with host buffers: every step uploads its input from
    # pinned host memory, applies the layer and downloads its result. With room for more
    # pinned state buffers, up to three registers on their own streams take turns as a
    # three-stage pipeline: uploads run one after another in issue order, so do the layers and
    # the downloads (cross-stream events), so one register's upload, another's layer and a
    # third's download overlap instead of splitting each engine between them. The copies are
    # SetStateVectorAsync / GetStateVectorAsync, queued in stream order with the gates.
    state_bytes = (1 << n) * 16
    avail = host_mem_available()
    nreg = 3 if avail >= 4 * state_bytes + (16 << 30) else (2 if avail >= 3 * state_bytes + (16 << 30) else 1)
    regs, hosts, streams = [reg], [], [stream]
    for _ in range(1, nreg):
        st_ = torch.cuda.Stream()
        r2 = iqs.QubitRegister(n, "", 0, math=args.math, stream=st_.cuda_stream)
        if args.width:
            r2.SetSweepWidth(args.width)
            r2.SetSweepPipeline(args.pipeline)
            if args.math == "emulated":
                r2.SetNativeShare(args.native_share)
        elif tuned:
            r2.SetSweepWidth(tuned["width"])
            r2.SetSweepPipeline(tuned["pipeline"])
            if args.math == "emulated":
                r2.SetNativeShare(tuned["native_share"])
        if args.fusion:
            r2.TurnOnFusion()
        regs.append(r2)
        streams.append(st_)
    for r_ in regs:
        h_ = torch.empty(1 << n, dtype=torch.complex128, pin_memory=True)  # the tensor keeps the pinned block
        reg.GetStateVector(out=h_.numpy())
        hosts.append(h_)
    e2e_steps = min(max(4 * nreg, args.steps), 12)
    last = {"up": None, "layer": None, "down": None}

    def stage(st_, key, fn):
        if last[key] is not None:
            st_.wait_event(last[key])
        fn()
        ev = torch.cuda.Event()
        ev.record(st_)
        last[key] = ev

    def e2e_step(i, s):
        r_, hb, st_ = regs[i], hosts[i], streams[i]

        def layer():
            apply_layer(r_, mats[s], n)
            r_.ApplyFusedGates()
        stage(st_, "up", lambda: r_.SetStateVectorAsync(hb.numpy()))     # host (pinned) -> HBM
        stage(st_, "layer", layer)
        stage(st_, "down", lambda: r_.GetStateVectorAsync(hb.numpy()))   # HBM -> host (pinned)

    for i_ in range(nreg):                            # untimed: first use of each buffer and stream
        e2e_step(i_, args.warmup)
    for r_ in regs:
        r_.synchronize()
    barrier()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        e2e_step(s % nreg, args.warmup + s % args.steps)
    for r_ in regs:
        r_.synchronize()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist)
    e2e_value = job_gbs(world, layer_bytes(n), e2e_s)
    del hosts
    del regs[1:]
    pipelined = nreg

    # Same layer with native FP64 arithmetic, for comparison (2 steps).
    other = {}
    if n >= 20 and args.compare_native and args.math == "emulated":
        reg.SetMath("native")
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for s in range(2):
            step(args.warmup + s % args.steps)
        b.record(stream)
        barrier()
        nat_ms = a.elapsed_time(b) / 2
        other = {"native_fp64": {"value": round(layer_bytes(n) / (nat_ms * 1e-3) / 1e9, 1), "ms_per_step": round(nat_ms, 3)}}
        reg.SetMath(args.math)

    del reg
    torch.cuda.synchronize()

    # Parity of the timed arithmetic on the same layer shape at 20 qubits vs the oracle.
    parity = None
    cpu = None
    qaoa = None
    batched = None
    qft = None
    trotter = None
    plain = None
    if rank == 0:
        import oracle
        oracle.build(ref=False)
        m20 = haar_layers(20, 2, seed=7)
        g = iqs.QubitRegister(20, "base", 0, math=args.math)
        if args.fusion:
            g.TurnOnFusion()
        o = oracle.OracleRegister(20, "base", 0)
        for r_ in (g, o):
            for q in range(20):
                r_.ApplyHadamard(q)
            for l in range(2):
                apply_layer(r_, m20[l], 20)
        parity = float(np.max(np.abs(g.GetStateVector() - o.GetStateVector())))
        del g
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            cpu = cpu_layer_gbs(args.cpu_qubits, 1, seed=5, threads=threads)
        qaoa = None if args.no_adjoint else qaoa_section(stream=stream.cuda_stream)
        batched = None if args.no_batched else batched_section()
        plain = plain_section()
        qft = None if args.no_qft else qft_brick_section()
        trotter = None if args.no_trotter else trotter_section(grad_steps=100 if args.full_trotter else 10)

    if rank == 0:
        dtype = ("c128: f64 amplitudes at every call boundary, double-float (fp32x2) products and sums"
                 + (", held as double-float pairs between the passes of a call" if df_runs else "")
                 if args.math == "emulated" else "f64")
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded Haar-random gates on a dense state)",
            "config": {"workload": f"gate layer: Haar U on each of {n} qubits + CZ brick ({n // 2} even + {(n - 1) // 2} odd), ComplexDP",
                       "qubits": n, "state_bytes": (1 << n) * 16, "bytes_per_step": layer_bytes(n),
                       "math": args.math, "fusion": bool(args.fusion),
                       "sweep_width": args.width or (tuned["width"] if tuned else "default"),
                       "sweep_pipeline": bool(args.pipeline if args.width else (tuned["pipeline"] if tuned else False)),
                       "native_share_16ths": (args.native_share if args.width else (tuned["native_share"] if tuned else 0))
                       if args.math == "emulated" else None,
                       "autotune_ms": [[r["width"], r["pipeline"], r["native_share"], round(r["ms"], 1)]
                                       for r in tuned["table"]] if tuned else None,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": f"state ({(1 << n) * 16 / 2**30:g} GiB) far larger than L2 (129 MB); no flush needed"},
            "roofline": {"bound": "hbm", "kernel": kname,
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_src,
                         "bytes_per_launch": 2 * (1 << n) * 16, "avg_launch_ms": round(k_avg, 4),
                         "traffic": traffic, "traffic_source": traffic_src},
            "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": (1 << n) * 16,
                    "d2h_bytes_per_step": (1 << n) * 16, "steps": e2e_steps,
                    "path": (f"{pipelined} registers on their own streams take turns as a three-stage pipeline "
                             "(uploads, layers and downloads each in issue order): " if pipelined > 1 else "") +
                            "QubitRegister.SetStateVectorAsync (pinned host) + layer via the public API + "
                            "GetStateVectorAsync (pinned host), wall clock over all steps"},
            "gpu_launches": launches,
            "sweeps": sweeps,
            "df_storage_runs": df_runs,
            "clocks": clk,
            "parity": {"max_abs_err_vs_oracle": parity, "case": "same layer shape at 20 qubits, 2 layers"},
        }
        line.update(other)
        if qaoa is not None:
            line["adjoint"] = qaoa
        if batched is not None:
            line["batched"] = batched
        if plain is not None:
            line["plain_gate_by_gate_20q"] = plain
        if qft is not None:
            line["qft_brick"] = qft
        if trotter is not None:
            line["trotter"] = trotter
        if cpu is not None:
            line["cpu_baseline"] = {"value": round(cpu["gbs"], 3), "unit": UNIT, "cores": cpu["cores"],
                                    "kind": cpu["kind"],
                                    "sample": f"one {args.cpu_qubits}-qubit layer (same layer shape), "
                                              f"{cpu['seconds']:.1f} s"}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--cpu-qubits", type=int, default=28)
    ap.add_argument("--math", choices=["emulated", "native"], default="emulated")
    ap.add_argument("--compare-native", action="store_true", default=True)
    ap.add_argument("--no-fusion", dest="fusion", action="store_false", default=True,
                    help="apply the layer gate by gate (one kernel per gate)")
    ap.add_argument("--width", type=int, default=0,
                    help="fused-pass width (target qubits per pass); 0 = chosen by the autotuner")
    ap.add_argument("--pipeline", type=int, default=0, help="with --width: 1 = bulk-copy pipelined passes")
    ap.add_argument("--native-share", type=int, default=0,
                    help="with --width and emulated math: sixteenths of the warps on native FP64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the QAOA adjoint-gradient section")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-circuits section")
    ap.add_argument("--no-qft", action="store_true", help="skip the QFT + brick-layers section")
    ap.add_argument("--no-trotter", action="store_true", help="skip the XXZ Trotter section")
    ap.add_argument("--full-trotter", action="store_true",
                    help="adjoint gradient over all 100 Strang steps at 32 qubits (about 1.5 min more)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="dram bytes per 1-qubit-gate launch from an ncu capture, if known")
    ap.add_argument("--only", choices=["plain", "adjoint", "batched", "qft", "trotter"], default=None,
                    help="run one section alone and print its JSON (a profiling entry point; not the bench line)")
    ap.add_argument("--section-qubits", type=int, default=0, help="with --only: register size of the section")
    ap.add_argument("--section-steps", type=int, default=0, help="with --only trotter: Strang steps")
    ap.add_argument("--tile-qubits", type=int, default=0,
                    help="with --only trotter: run the ComplexSP chain as shared-memory tile passes of this size")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.only:
        run_section(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


def run_section(args) -> None:
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    q, st = args.section_qubits, args.section_steps
    if args.only == "plain":
        out = plain_section()
    elif args.only == "adjoint":
        out = qaoa_section(n=q or 26)
    elif args.only == "batched":
        out = batched_section(count=q or 4096)
    elif args.only == "qft":
        out = qft_brick_section(n=q or 30)
    else:
        out = trotter_section(n=q or 32, steps=st or 100, n_dp=(q + 1) if q else 33, steps_dp=4,
                              grad_steps=min(st or 10, 10), tile_qubits=args.tile_qubits)
    print(json.dumps({"section": args.only, **out}), flush=True)


if __name__ == "__main__":
    main()
