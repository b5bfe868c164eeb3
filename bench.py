"""Benchmark of the CQBEM Laplace-domain assembly on GB300.

Workload (default): the mixed-size object set -- 24 objects, icospheres with 162/642/2562 vertices
drawn with probabilities 0.5/0.35/0.15, scaled to seeded ellipsoids (axes 0.5-2 x 0.1 m), E
log-uniform in [1e4, 1e6] Pa, nu uniform in [0.2, 0.45], rho 1000, dt = 1/200, BDF2, N in {16, 32}
(L = N + 1, L/2 + 1 Laplace frequencies), collocation with the 7-point rule.  Synthetic and seeded;
the reference publishes no dataset or numbers for this path.

One step = every Laplace-domain matrix (G, H, B_trans, B_angular at every frequency) of every
object.  Metric: complex matrix entries per second, counted as sum over objects of
(L/2+1) * (2 (3V)^2 + 12 * 3V).

  value : device-resident path -- the batched persistent kernels of all objects and frequencies
          under one CUDA graph, outputs complex64 kept in HBM; CUDA-event time over K steps, L2
          flushed between steps.
  e2e   : the drop-in through the C ABI with host buffers -- one sod_cqbem_assemble_all call per
          object, the replacement of the frequency loops of compute_{G,H,B_trans,B_angular}_matrices,
          into pinned host arrays of every frequency in the reference layout (complex128), timed end
          to end (row chunks copied to the host while later rows compute).  The CPU-GPU link bounds
          it: ~193 GB/s device to host on GB300, by copy engine or by mapped stores alike.
  --impl reference : the reference's CPU algorithm (the oracle's reference-mixed restatement,
          OpenMP on all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic FP32 flops per kernel evaluation (field point x quadrature point x frequency),
# regular collocation pass: geometry + two complex exponentials + kernel combination
FLOPS_PER_EVAL = {"G": 130, "H": 240, "B_trans": 60, "B_angular": 150}
# per batched pass: the G scatter also integrates B_trans and B_angular from the same radial terms
# (130 + 60 + 150); the stand-alone B reduction (batches without G) does 60 + 150
PASS_FLOPS = {"scatter_G": 340, "scatter_H": 240, "reduce_B": 210}
# DRAM bytes per evaluation of each pass from an ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum over the launch's evaluations): the capture of the 2562-vertex scatter pair at two
# frequencies (183.4 M evaluations per launch: 897 MB and 892 MB, almost all of it the complex64 output rows)
TRAFFIC_BYTES_PER_EVAL = {"scatter_G": 4.89, "scatter_H": 4.87}
KINDS = ("G", "H", "B_trans", "B_angular")


def make_workload(seed: int = 2024, n_objects: int = 24):
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    rng = np.random.default_rng(seed)
    objs = []
    for k in range(n_objects):
        level = int(rng.choice([2, 3, 4], p=[0.5, 0.35, 0.15]))
        axes = rng.uniform(0.5, 2.0, size=3)
        E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        nu = float(rng.uniform(0.2, 0.45))
        N = int(rng.choice([16, 32]))
        mesh = make_icosphere_mesh(level, 0.1, axes=axes, seed=seed + k)
        objs.append(dict(mesh=mesh, mat=Material(E, nu, 1000.0), N=N, dt=1.0 / 200.0, bdf=2, order=5, subdiv=1))
    return objs


def make_single(level: int = 3):
    """One object: icosphere radius 0.1 m, E 1e5, nu 0.3, rho 1000, dt 0.01, BDF2, N 32, 7-point rule
    (the reference's CPU-runnable collocation case at level 3: 642 vertices / 1280 triangles)."""
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    return [dict(mesh=make_icosphere_mesh(level, 0.1), mat=Material(1e5, 0.3, 1000.0), N=32, dt=0.01, bdf=2,
                 order=5, subdiv=1)]


def make_single_2f():
    """The 2562-vertex object of make_single(4) with two of its 17 frequencies (l = 4 and 12): the
    scatter kernels at full mesh size with ~2 GB of outputs, small enough for an ncu --set full capture."""
    objs = make_single(4)
    objs[0]["fsel"] = (4, 12)
    return objs


CASES = {"mixed24": make_workload, "coll642": lambda: make_single(3), "coll2562": lambda: make_single(4),
         "coll162": lambda: make_single(2), "coll2562_2f": make_single_2f}


def entries(nV: int, nfreq: int) -> int:
    return nfreq * (2 * (3 * nV) ** 2 + 12 * 3 * nV)


def kind_entries(kind: str, nV: int) -> int:
    """complex entries of one frequency of one kind: 3V x 3V (G, H), 3V x 3, 3V x 9"""
    return {"G": (3 * nV) ** 2, "H": (3 * nV) ** 2, "B_trans": 9 * nV, "B_angular": 27 * nV}[kind]


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
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
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measure_fp32_peak(torch, dev) -> float:
    """cuBLAS SGEMM with TF32 disabled (FP32 CUDA-core pipes), best of 5, TFLOP/s."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev, dtype=torch.float32)
    b = torch.randn(n, n, device=dev, dtype=torch.float32)
    for _ in range(2):
        torch.mm(a, b)
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    return best


def cpu_sample(objs, threads: int, freqs_per_object: int = 3, seed: int = 29):
    """Reference CPU path (oracle, reference-mixed precision, OpenMP over field vertices) on a bounded,
    stratified sample of the whole workload: every object and every kind, `freqs_per_object` of the
    object's frequencies (spread over its list: first, middle and last for three) and a seeded subset of
    2 x threads field vertices (all of them on smaller meshes).  A stratum's (object, kind) time is
    scaled by its row and frequency sampling fractions to estimate the CPU time of the whole step (the
    per-entry cost of a row does not depend on the row or on the frequency); returns the workload's
    entries / that estimate, the sample's wall time, the cores, a description and the estimate."""
    from oracle import oracle as O

    O.build()
    cores = O.set_threads(threads)
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    est, total, calls = 0.0, 0, 0
    for obj in objs:
        m, mat = obj["mesh"], obj["mat"]
        s, R, L = O.cq_frequencies(obj["bdf"], obj["dt"], obj["N"])
        if "fsel" in obj:
            s = s[list(obj["fsel"])]
        nf = len(s)
        pick = sorted(set(np.linspace(0, nf - 1, max(1, min(freqs_per_object, nf))).round().astype(int).tolist()))
        nr = min(m.nV, 2 * cores)
        rows = np.sort(rng.choice(m.nV, nr, replace=False)).astype(np.int32)
        for kind in KINDS:
            total += nf * kind_entries(kind, m.nV)
            t1 = time.perf_counter()
            for l in pick:
                O.collocation(kind, m, mat, s[l], order=obj["order"], subdiv=obj["subdiv"], rows=rows, mode=O.MIXED)
                calls += 1
            est += (time.perf_counter() - t1) * (m.nV / nr) * (nf / len(pick))
    dt = time.perf_counter() - t0
    sample = (f"stratified: all {len(objs)} objects x 4 kinds, {freqs_per_object} frequencies per object, "
              f"{2 * cores} seeded field vertices per object (all on smaller meshes); {calls} calls in "
              f"{dt:.1f} s; whole-step CPU time estimated from the strata at {est:.0f} s")
    return total / est, dt, cores, sample, est


def check_batched_rows(objs, outs, rows_per_object: int = 2, seed: int = 17) -> dict:
    """Relative Frobenius error of the batched step's device outputs on sampled rows (seeded field
    vertices of every object) at the first, middle and last frequency, against the FP64 oracle's
    row-sampled assembly (those rows are exact: every face is integrated for the listed vertices)."""
    from oracle import oracle as O

    O.build()
    rng = np.random.default_rng(seed)
    num = {k: 0.0 for k in KINDS}
    den = {k: 0.0 for k in KINDS}
    worst = {k: 0.0 for k in KINDS}
    for o, per in zip(objs, outs):
        m = o["mesh"]
        rows = np.sort(rng.choice(m.nV, size=min(rows_per_object, m.nV), replace=False)).astype(np.int32)
        idx = np.concatenate([np.arange(3 * v, 3 * v + 3) for v in rows])
        nf = len(o["s"])
        for l in sorted({0, nf // 2, nf - 1}):
            for kind in KINDS:
                got = per[kind][l].cpu().numpy()[idx].astype(np.complex128)
                ref = O.collocation(kind, m, o["mat"], o["s"][l], order=o["order"], subdiv=o["subdiv"], rows=rows)
                d, r = float(np.linalg.norm(got - ref)), float(np.linalg.norm(ref))
                num[kind] += d * d
                den[kind] += r * r
                worst[kind] = max(worst[kind], d / r)
    return {"check": f"{rows_per_object} seeded rows per object, first / middle / last frequency, vs FP64 oracle rows",
            "rel_err_stacked": {k: (num[k] / den[k]) ** 0.5 for k in KINDS}, "rel_err_worst": worst,
            "tolerance": 1e-5}


def measured_hbm_gbs() -> float:
    """HBM copy bandwidth measured on the GB300s (MEASURED_PEAKS.json), else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def history_leg(torch, ctx, stream, n: int = 7686, K: int = 64, reps: int = 10):
    """Per-step history convolution of one 2562-vertex object (3V = 7686), N = 64 weights of G and H:
    FP32 and BF16 (+ per-row scales) banks, 1 and 16 right-hand sides.  Inputs resident in HBM;
    weights far larger than L2.  Algorithmic bytes = the bank's weight bytes per step."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    hbm = measured_hbm_gbs()
    rows = []
    cases = [(L.F32, "f32", 1, "cuda_cores"), (L.F32, "f32", 16, "tensor_cores"), (L.F32, "f32", 16, "cuda_cores"),
             (L.BF16, "bf16", 1, "tensor_cores"), (L.BF16, "bf16", 1, "cuda_cores"), (L.BF16, "bf16", 16, "tensor_cores"),
             (L.BF16, "bf16", 16, "cuda_cores")]
    for wdt, name, R, engine in cases:
        bank = api.HistoryBank(ctx, n, n, K, R, wdt)
        bank.set_engine(L.HISTORY_ENGINE_TENSOR_CORES if engine == "tensor_cores" else L.HISTORY_ENGINE_CUDA_CORES)
        g = torch.empty((n, n), dtype=torch.float32, device="cuda")
        gen = torch.Generator(device="cuda")
        gen.manual_seed(7)
        for k in range(1, K + 1):
            g.normal_(0.0, 0.8 ** k, generator=gen)
            bank.set_weights(k, g, g)
        shape = (n, R) if R > 1 else (n,)
        for _ in range(K):
            t = torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen) * 10.0
            d = torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen) * 1e-4
            bank.push(t, d)
        out = torch.empty(shape, dtype=torch.float64, device="cuda")
        for _ in range(3):
            bank.convolve(out)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bank.convolve(out)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts))
        wb = bank.weight_bytes
        rows.append({"weights": name, "rhs": R, "engine": engine, "ms": round(ms, 4),
                     "gb_per_s": round(wb / ms / 1e6, 1), "hbm_frac": round(wb / ms / 1e6 / hbm, 4), "bytes": wb,
                     "tflops": round(4.0 * K * n * n * R / ms / 1e9, 2)})
        bank.close()
        del g, out
        torch.cuda.empty_cache()
    # wavelet-compressed bank (Haar non-standard form, 10% of the 9 nV^2 coefficients kept per matrix,
    # the ratio of the reference's compressed-history scenes)
    rows.append(wavelet_case(torch, ctx, stream, n // 3, K, 0.1, reps, hbm))
    return {"object": "3V = 7686 (2562 vertices), N = 64", "peak_gbs": hbm,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth, measured)", "cases": rows}


def wavelet_case(torch, ctx, stream, nV: int, K: int, ratio: float, reps: int, hbm: float) -> dict:
    """Per-step convolution of a wavelet-compressed bank (3 nV rows, K steps, `ratio` of the
    coefficients kept), synthetic FP32 weights as the dense cases; algorithmic bytes = the kept
    coefficients x 12 B (FP64 value + packed column)."""
    import time

    from surfaceonlydeformables_gb300 import api

    n = 3 * nV
    bank = api.HistoryBank.compressed(ctx, nV, K, ratio)
    g = torch.empty((n, n), dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(1, K + 1):
        g.normal_(0.0, 0.8 ** k, generator=gen)
        bank.set_weights(k, g, g)
    for _ in range(K):
        bank.push(torch.randn(n, dtype=torch.float64, device="cuda", generator=gen) * 10.0,
                  torch.randn(n, dtype=torch.float64, device="cuda", generator=gen) * 1e-4)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    bank.convolve(out)  # merges the blocks
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    for _ in range(3):
        bank.convolve(out)
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bank.convolve(out)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    ms = float(np.median(ts))
    wb = bank.weight_bytes
    bank.close()
    del g, out
    torch.cuda.empty_cache()
    return {"weights": f"haar_ratio_{ratio}", "rows": n, "K": K, "rhs": 1, "engine": "sparse_cuda_cores",
            "ms": round(ms, 4), "gb_per_s": round(wb / ms / 1e6, 1), "hbm_frac": round(wb / ms / 1e6 / hbm, 4),
            "bytes": wb, "setup_s": round(setup_s, 2)}


def scenes_leg(torch, ctx, stream):
    """The reference's own scenes (meshes from tests/golden): the time-domain precompute of the cube
    scene (data/cube_drop.json: 870-vertex traction-discontinuous cube, mu 1e5, nu 0.45, rho 1000,
    BDF1, dt 0.005, order 5 / subdivision 2, N = 6) and of the bunny scene (data/bunny_friction.json:
    3485 vertices, mu 1e6, nu 0.3, rho 3000, BDF1, dt 0.003, N = 5), device-resident FP64 outputs,
    and one step of their wavelet-compressed histories at the scenes' ratio 0.1 (cube_collide,
    bunny_friction).  Event-timed second runs (the first builds the mesh schedules)."""
    import os

    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import Material, SurfaceMesh

    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden")
    cube = np.load(os.path.join(golden, "cube_meshes.npz"))
    bunny = np.load(os.path.join(golden, "bunny_mesh.npz"))
    scenes = [("cube_drop", SurfaceMesh.from_arrays(cube["V_disc"], cube["F_disc"]), cube["vmap_disc"],
               Material(2.0 * 1e5 * (1.0 + 0.44999998807907104), 0.44999998807907104, 1000.0), 0.004999999888241291, 6),
              ("bunny_friction", SurfaceMesh.from_arrays(bunny["V"], bunny["F"]), None,
               Material(2.0 * 1e6 * 1.3, 0.3, 3000.0), 0.003, 5)]
    res = {}
    for name, mesh, vmap, mat, dt, N in scenes:
        dm = api.Mesh(ctx, mesh, vmap=vmap)

        def run():
            return api.precompute(ctx, dm, mat, 1, dt, N, order=5, subdiv=2)

        w = run()
        del w
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w = run()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        n3 = 3 * mesh.nV
        lam = (N + 1) // 2 + 1
        entries = lam * (2 * n3 * n3 + 12 * n3)
        out = {"vertices": mesh.nV, "faces": mesh.nF, "N": N, "precompute_ms": round(ms, 2),
               "laplace_entries_per_s": entries / (ms * 1e-3)}
        bank = api.HistoryBank.compressed(ctx, mesh.nV, N, 0.1)
        for k in range(1, N + 1):
            bank.set_weights(k, w["G"][k], w["H"][k])
        gen = torch.Generator(device="cuda")
        gen.manual_seed(1)
        for _ in range(N):
            bank.push(torch.randn(n3, dtype=torch.float64, device="cuda", generator=gen),
                      torch.randn(n3, dtype=torch.float64, device="cuda", generator=gen))
        b = torch.empty(n3, dtype=torch.float64, device="cuda")
        for _ in range(3):
            bank.convolve(b)
        torch.cuda.synchronize()
        e0.record(stream)
        bank.convolve(b)
        e1.record(stream)
        torch.cuda.synchronize()
        out["compressed_history_step_ms"] = round(e0.elapsed_time(e1), 4)
        out["compressed_history_bytes"] = bank.weight_bytes
        bank.close()
        del w, b
        dm.close()
        torch.cuda.empty_cache()
        res[name] = out
    return res


def precompute_leg(torch, ctx, stream, levels=(3, 4)):
    """Time-domain precompute (sod_cqbem_precompute: every Laplace frequency of G, H, B_trans, B_angular
    with the compensated regular pass, the inverse transform, the free term, B_euler) of one icosphere:
    level 3 is the single-object case (642 vertices, E 1e5, nu 0.3, dt 0.01, BDF2, N 32), level 4 the
    2562-vertex object at the same parameters.  Device-resident FP64 outputs.  Time-domain entries =
    L (2 (3V)^2 + 6 3V) (G, H, and B = [B_trans | B_euler]); B_angular's 27 per row ride along.  The
    same call with the regular pass in FP32 is timed beside it (its late weights are not accurate)."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    res = {}
    for level in levels:
        m = make_icosphere_mesh(level, 0.1)
        dm = api.Mesh(ctx, m)
        mat = Material(1e5, 0.3, 1000.0)
        N = 32
        n3 = 3 * m.nV
        row = {"vertices": m.nV, "N": N}
        for prec, tag in ((L.PRECISION_AUTO, "compensated"), (L.PRECISION_FP32, "fp32_regular_pass")):
            ctx.set_precision(prec)
            w = api.precompute(ctx, dm, mat, 2, 0.01, N)
            del w
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            w = api.precompute(ctx, dm, mat, 2, 0.01, N)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            del w
            torch.cuda.empty_cache()
            row[tag] = {"ms": round(ms, 2), "time_domain_entries_per_s": (N + 1) * (2 * n3 * n3 + 6 * n3) / (ms * 1e-3)}
        ctx.set_precision(L.PRECISION_AUTO)
        dm.close()
        res[f"ico{m.nV}"] = row
    return res


def elastostatic_leg(torch, ctx, stream):
    """Elastostatic Kelvin G and H (H with the rigid-mode diagonal correction) of the 2562-vertex
    object, device-resident FP64 output."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    m = make_icosphere_mesh(4, 0.1, jitter=0.2, seed=11)
    dm = api.Mesh(ctx, m)
    mat = Material(1e5, 0.45, 1000.0)
    out = torch.empty((3 * m.nV, 3 * m.nV), dtype=torch.float64, device="cuda")
    res = {}
    for method, tag in ((L.COLLOCATION, ""), (L.GALERKIN, "galerkin_")):
        for kind in ("G", "H"):
            api.elastostatic(ctx, dm, kind, mat, method=method, out=out)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            api.elastostatic(ctx, dm, kind, mat, method=method, out=out)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            res[tag + kind] = {"ms": round(ms, 3), "entries_per_s": (3 * m.nV) ** 2 / (ms * 1e-3)}
    return {"mesh": f"icosphere level 4, {m.nV} vertices, jittered", "rule": "7-point regular, singular order 5", **res}


def solve_leg(torch, ctx, stream, n: int = 7686, K: int = 8):
    """Dense FP64 solves of the 2562-vertex object's size (3V = 7686): the H_0 LU, u_p = H_0^-1 G'
    (3V right-hand sides), the explicit inverse, and one served step u = H_0^-1 b fused after a
    K-step FP32 history convolution (1 and 16 right-hand sides).  Synthetic, well-conditioned
    matrices of that size stand in for H_0 and G'."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    A = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen) + n ** 0.5 * torch.eye(
        n, dtype=torch.float64, device="cuda")
    G = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen)

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), r

    try:
        api.Solver(ctx, torch.eye(8, dtype=torch.float64, device="cuda")).close()  # library load, handles
        ms_lu_first, S = timed(lambda: api.Solver(ctx, A))  # includes first-use kernel loading
        S.close()
        ms_lu, S = timed(lambda: api.Solver(ctx, A))
    except L.SodError as e:
        return {"unavailable": str(e)}
    X = torch.empty_like(G)
    S.solve(G, out=X)
    ms_up, _ = timed(lambda: S.solve(G, out=X))
    ms_inv, _ = timed(lambda: S.inverse(out=X))
    res = {"n": n, "lu_ms": round(ms_lu, 2), "lu_first_ms": round(ms_lu_first, 2),
           "lu_tflops_fp64": round(2 / 3 * n ** 3 / ms_lu / 1e9, 3),
           "u_p_solve_ms": round(ms_up, 2), "inverse_ms": round(ms_inv, 2)}
    del X, G
    for R in (1, 16):
        bank = api.HistoryBank(ctx, n, n, K, R, L.F32)
        w = torch.empty((n, n), dtype=torch.float32, device="cuda")
        for k in range(1, K + 1):
            w.normal_(0.0, 0.8 ** k, generator=gen)
            bank.set_weights(k, w, w)
        shape = (n, R) if R > 1 else (n,)
        for _ in range(K):
            bank.push(torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen),
                      torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen))
        out = torch.empty(shape, dtype=torch.float64, device="cuda")
        bank.convolve_solve(S, out)
        ms_c, _ = timed(lambda: bank.convolve(out))
        ms_cs, _ = timed(lambda: bank.convolve_solve(S, out))
        res[f"step_rhs{R}"] = {"convolve_ms": round(ms_c, 3), "convolve_lu_solve_ms": round(ms_cs, 3)}
        bank.close()
        del w, out
    S.keep_inverse()
    for R in (1, 16):
        bank = api.HistoryBank(ctx, n, n, K, R, L.F32)
        w = torch.empty((n, n), dtype=torch.float32, device="cuda")
        for k in range(1, K + 1):
            w.normal_(0.0, 0.8 ** k, generator=gen)
            bank.set_weights(k, w, w)
        shape = (n, R) if R > 1 else (n,)
        for _ in range(K):
            bank.push(torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen),
                      torch.randn(shape, dtype=torch.float64, device="cuda", generator=gen))
        out = torch.empty(shape, dtype=torch.float64, device="cuda")
        bank.convolve_solve(S, out)
        ms_ci, _ = timed(lambda: bank.convolve_solve(S, out))
        res[f"step_rhs{R}"]["convolve_inverse_gemv_ms"] = round(ms_ci, 3)
        bank.close()
        del w, out
    S.close()
    # B_trans_inv.solve(H_0): minimum-norm least squares with a tall 3V x 3 matrix (one pass over Y)
    Bt = torch.randn((n, 3), dtype=torch.float64, device="cuda", generator=gen)
    Y = torch.randn((n, n), dtype=torch.float64, device="cuda", generator=gen)
    X3 = torch.empty((3, n), dtype=torch.float64, device="cuda")
    ms_f, C = timed(lambda: api.LeastSquares(ctx, Bt))
    C.solve(Y, out=X3)
    ms_s, _ = timed(lambda: C.solve(Y, out=X3))
    res["lstsq_3col"] = {"factor_ms": round(ms_f, 3), "solve_ms": round(ms_s, 3),
                         "solve_gbs": round(n * n * 8 / ms_s / 1e6, 1)}
    C.close()
    del Y, X3
    if n % 3 == 0 and n // 3 in (12, 42, 162, 642, 2562):
        # elastostatic u_p from the icosphere's own Kelvin H and G (collocation)
        from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

        level = (12, 42, 162, 642, 2562).index(n // 3)
        dm = api.Mesh(ctx, make_icosphere_mesh(level, 0.1))
        mat = Material(1e5, 0.3, 1000.0)
        H = torch.empty((n, n), dtype=torch.float64, device="cuda")
        Gs = torch.empty_like(H)
        api.elastostatic(ctx, dm, "H", mat, out=H)
        api.elastostatic(ctx, dm, "G", mat, out=Gs)
        up = torch.empty_like(H)
        ms_up2, _ = timed(lambda: api.elastostatic_u_p(ctx, dm, H, Gs, out=up))
        flop = 2 * n ** 3 + n ** 3 + n ** 3 / 3 + 2 * n ** 3  # GEMM, SYRK, Cholesky, n-RHS solve
        res["elastostatic_u_p"] = {"ms": round(ms_up2, 1), "fp64_tflops": round(flop / ms_up2 / 1e9, 3)}
        dm.close()
        del H, Gs, up
    return res


def galerkin_leg(torch, ctx, stream, nfreq: int | None = None, level: int = 4):
    """Galerkin G and H of the jittered icosphere (level 4 = 2562 vertices, the Galerkin case: E 1e5, nu 0.45,
    dt 1/200, N = 64 -> 33 Laplace frequencies; 13-point rule for regular pairs, Sauter-Schwab order 5
    for the singular ones), timed over all 33 frequencies (or `nfreq` of them, from l = 1), with four
    rows of the first and the last timed frequency checked against the FP64 oracle (the rows of the
    listed vertices are exact in the row-sampled oracle).  Level 3 (642 vertices) is the small case
    for profiling captures."""
    from oracle import oracle as O

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    m = make_icosphere_mesh(level, 0.1, jitter=0.2, seed=2)
    rows = (0, m.nV // 5, m.nV // 2, m.nV - 1)
    dm = api.Mesh(ctx, m)
    mat = Material(1e5, 0.45, 1000.0)
    s, R, Lq = L.cq_frequencies(2, 1 / 200, 64)
    nfreq = len(s) if nfreq is None or nfreq >= len(s) else nfreq
    sel = s if nfreq == len(s) else s[1:1 + nfreq]
    n = 3 * m.nV
    out = {k: torch.empty((nfreq, n, n), dtype=torch.complex64, device="cuda") for k in ("G", "H")}
    api.assemble_frequencies(ctx, dm, "G", mat, sel[:1], order=7, sorder=5, ssub=1, method=L.GALERKIN,
                             out=out["G"][:1], dtype=L.C64)
    torch.cuda.synchronize()
    res = {}
    for kind in ("G", "H"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        api.assemble_frequencies(ctx, dm, kind, mat, sel, order=7, sorder=5, ssub=1, method=L.GALERKIN,
                                 out=out[kind], dtype=L.C64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        O.build()
        r = np.array(rows, dtype=np.int32)
        idx = np.concatenate([np.arange(3 * v, 3 * v + 3) for v in r])
        errs = []
        for l in sorted({0, nfreq - 1}):
            got = out[kind][l].cpu().numpy()[idx]
            ref = O.galerkin(kind, m, mat, sel[l], order=7, sorder=5, ssub=1, rows=r)
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
        res[kind] = {"ms": round(ms, 2), "ms_per_frequency": round(ms / nfreq, 2),
                     "entries_per_s": n * n * nfreq / (ms * 1e-3), "rel_err_vs_fp64_rows": max(errs)}
    del out
    torch.cuda.empty_cache()
    return {"mesh": f"icosphere level {level} jittered (sigma 0.2 edge), {m.nV} vertices / {m.nF} faces",
            "frequencies_timed": f"{nfreq} of {len(s)}", "rule": "13-point regular, Sauter-Schwab order 5",
            "oracle_rows": list(rows), **res}


def serving_requests(seed: int, n_requests: int, rate_hz: float):
    """Poisson arrivals; 30% assembly requests (objects from the mixed-size distribution), 70% time
    steps of device-resident objects with seeded Gaussian tractions (10 Pa) and displacements.  A step
    targets one of the 4 most recently submitted objects: 4 banks of the largest class (15.6 GB each)
    plus the two assemblies in flight (31 GB each with their transform buffers) stay under the 150 GB
    cap, so the targets stay resident under least-recently-used eviction."""
    from surfaceonlydeformables_gb300.meshes import Material, make_icosphere_mesh

    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    objs = []
    for k in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        if not objs or rng.random() < 0.3:
            level = int(rng.choice([2, 3, 4], p=[0.5, 0.35, 0.15]))
            axes = rng.uniform(0.5, 2.0, size=3)
            E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
            nu = float(rng.uniform(0.2, 0.45))
            N = int(rng.choice([16, 32]))
            mesh = make_icosphere_mesh(level, 0.1, axes=axes, seed=seed + k)
            objs.append(len(reqs))
            reqs.append(dict(t=t, type="assembly", mesh=mesh, mat=Material(E, nu, 1000.0), N=N))
        else:
            recent = objs[-4:]
            j = recent[int(rng.integers(len(recent)))]
            n = 3 * reqs[j]["mesh"].nV
            reqs.append(dict(t=t, type="step", target=j, p=rng.normal(size=n) * 10.0, u=rng.normal(size=n) * 1e-4))
    return reqs


def serving_leg(torch, ctx, n_requests: int = 240, rate_hz: float = 30.0, cap_gb: float = 150.0, seed: int = 99,
                per_object: bool | None = None):
    """Request loop (continuous batching, HBM-cap admission) against the plain drop-in on the same
    request stream (one request at a time, in arrival order).  The plain drop-in assembles an object
    as the reference's matrix collection does: one call per (kind, Laplace frequency) -- the
    per-frequency drop-in of the reference's per-row kernels -- with the compensated regular pass,
    then the inverse transform, then the history bank.  The per-object precompute (all frequencies
    of G and H in one call) is timed on the same stream as a second baseline."""
    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    reqs = serving_requests(seed, n_requests, rate_hz)

    def summary(lat, t_total, n_asm_entries):
        out = {}
        for ty in ("assembly", "step"):
            v = np.array([l for r, l in zip(reqs, lat) if r["type"] == ty and l is not None]) * 1e3
            if len(v):
                out[ty] = {"n": int(len(v)), "p50_ms": round(float(np.percentile(v, 50)), 3),
                           "p99_ms": round(float(np.percentile(v, 99)), 3)}
        out["requests_per_s"] = round(len(reqs) / t_total, 2)
        out["assembly_laplace_entries_per_s"] = n_asm_entries / t_total
        out["seconds"] = round(t_total, 2)
        return out

    def laplace_entries(r):
        n = 3 * r["mesh"].nV
        return (r["N"] // 2 + 1) * 2 * n * n  # G and H at every Laplace frequency

    asm_entries = sum(laplace_entries(r) for r in reqs if r["type"] == "assembly")

    # served: submit at the arrival times, collect completions
    srv = api.Server(0, int(cap_gb * (1 << 30)), 2, 2562)
    rid = [None] * len(reqs)
    t0 = time.perf_counter()
    for k, r in enumerate(reqs):
        while time.perf_counter() - t0 < r["t"]:
            time.sleep(0.0002)
        if r["type"] == "assembly":
            rid[k] = srv.submit_assembly(r["mesh"], r["mat"], 2, 1 / 200, r["N"])
        else:
            rid[k] = srv.submit_step(rid[r["target"]], r["p"], r["u"])
    srv.drain(3600)
    t_served = time.perf_counter() - t0
    done = {i: (st, lat) for i, st, lat in srv.poll(1 << 20)}
    lat_served = [done[i][1] * 1e-9 if done[i][0] == 0 else None for i in rid]
    n_failed = sum(1 for i in rid if done[i][0] != 0)
    srv.close()

    def plain_run(assemble_object):
        banks = {}  # insertion / use order = LRU order; evicted beyond the same HBM cap
        lat = [None] * len(reqs)
        cap = cap_gb * (1 << 30)
        t0 = time.perf_counter()
        for k, r in enumerate(reqs):
            now = time.perf_counter() - t0
            if now < r["t"]:
                time.sleep(r["t"] - now)
            if r["type"] == "assembly":
                n = 3 * r["mesh"].nV
                need = 8 * (r["N"] + 1) * n * n + 8 * r["N"] * n * ((n + 7) // 8 * 8)
                while banks and sum(b.weight_bytes for b in banks.values()) + need > cap:
                    banks.pop(next(iter(banks))).close()
                banks[k] = assemble_object(r)
            elif r["target"] in banks:
                bank = banks.pop(r["target"])
                banks[r["target"]] = bank  # most recently used
                bank.push(r["p"], r["u"])
                bank.convolve()
            else:
                continue  # evicted: the served loop reports these as failed requests too
            lat[k] = time.perf_counter() - t0 - r["t"]
        t = time.perf_counter() - t0
        for b in banks.values():
            b.close()
        torch.cuda.empty_cache()
        return lat, t

    def per_frequency(r):
        n = 3 * r["mesh"].nV
        s, R, Lq = L.cq_frequencies(2, 1 / 200, r["N"])
        m = api.Mesh(ctx, r["mesh"])
        ctx.set_precision(L.PRECISION_COMPENSATED)
        xhat = torch.empty((len(s), n, n), dtype=torch.complex128, device="cuda")
        w = {}
        for kind in ("G", "H"):
            for l, sl in enumerate(s):
                api.assemble(ctx, m, kind, r["mat"], sl, out=xhat[l])
            w[kind] = torch.empty((Lq, n, n), dtype=torch.float32, device="cuda")
            api.inverse_transform(ctx, xhat, Lq, R, out=w[kind], out_dtype=L.F32)
        ctx.set_precision(L.PRECISION_AUTO)
        bank = api.HistoryBank(ctx, n, n, r["N"], 1, L.F32)
        for i in range(1, r["N"] + 1):
            bank.set_weights(i, w["G"][i], w["H"][i])
        torch.cuda.synchronize()
        del xhat, w, m
        torch.cuda.empty_cache()
        return bank

    def whole_object(r):
        n = 3 * r["mesh"].nV
        m = api.Mesh(ctx, r["mesh"])
        pre = api.precompute(ctx, m, r["mat"], 2, 1 / 200, r["N"], kinds=("G", "H"), out_dtype=L.F32)
        bank = api.HistoryBank(ctx, n, n, r["N"], 1, L.F32)
        for i in range(1, r["N"] + 1):
            bank.set_weights(i, pre["G"][i], pre["H"][i])
        torch.cuda.synchronize()
        del pre, m
        torch.cuda.empty_cache()
        return bank

    lat_plain, t_plain = plain_run(per_frequency)
    out = {"requests": len(reqs), "arrivals": f"Poisson, {rate_hz} req/s, seed {seed}",
           "mix": "30% assembly (mixed-size set distribution, N in {16, 32}), 70% steps of submitted objects",
           "hbm_cap_gb": cap_gb, "assembly_slots": 2, "failed": n_failed,
           "served": summary(lat_served, t_served, asm_entries),
           "plain_drop_in": {"path": "per (kind, frequency) assembly calls, compensated regular pass, then the "
                                     "inverse transform and the bank, one request at a time",
                             **summary(lat_plain, t_plain, asm_entries)}}
    if per_object is None:
        per_object = n_requests <= 2000  # long runs: served against the plain drop-in only
    if per_object:
        lat_obj, t_obj = plain_run(whole_object)
        out["per_object_precompute"] = {"path": "sod_cqbem_precompute per object (all frequencies of G and H in "
                                                "one call), one request at a time",
                                        **summary(lat_obj, t_obj, asm_entries)}
    out["served_over_plain"] = round(t_plain / t_served, 3)
    return out


def max_over_ranks(torch, t_local: float, dist, device) -> float:
    """The job's time: every rank's timed-region seconds, reduced by max after a barrier (replicas
    run independently; the slowest sets the whole-job rate).  `dist` is torch.distributed or None."""
    t = torch.tensor([t_local], dtype=torch.float64, device=device)
    if dist:
        dist.barrier()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    objs = CASES[args.case]()
    threads = os.cpu_count() or 1
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    rates = []
    for it in range(args.warmup + args.steps):
        r, dt, cores, sample, est = cpu_sample(objs, threads)
        if it >= args.warmup:
            rates.append((r, dt, est))
    value = float(np.mean([r for r, _, _ in rates]))
    ms = float(np.mean([d for _, d, _ in rates]) * 1e3)  # the sample's wall time per step
    line = {"metric": "CQBEM Laplace-domain entries/s (mixed-size 24-object set)", "value": value,
            "unit": "entries/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32+fp64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "mixed-size 24-object collocation assembly (G,H,B_trans,B_angular, all "
                                   "Laplace frequencies); reference CPU path (oracle port, reference-mixed "
                                   "precision, OpenMP over field vertices), stratified sample",
                       "objects": len(objs), "vertices": [o["mesh"].nV for o in objs],
                       "frequencies": [len(o["fsel"]) if "fsel" in o else (o["N"] + 1) // 2 + 1 for o in objs],
                       "quadrature": "7-point (order 5), singular 5x5 FP64"},
            "cpu_baseline": {"value": value, "unit": "entries/s", "cores": cores, "kind": "port", "sample": sample,
                             "estimated_step_s": float(np.mean([e for _, _, e in rates]))},
            "e2e": {"value": value, "unit": "entries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch

    from surfaceonlydeformables_gb300 import _lib as L
    from surfaceonlydeformables_gb300 import api

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from surfaceonlydeformables_gb300 import build as B

    B.build()
    objs = CASES[args.case]()
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = api.Context(local, stream=stream)
    meshes = [api.Mesh(ctx, o["mesh"]) for o in objs]
    freqs = []
    for o in objs:
        s, R, Lq = L.cq_frequencies(o["bdf"], o["dt"], o["N"])
        if "fsel" in o:
            s = s[list(o["fsel"])].copy()
        o["s"], o["R"], o["L"] = s, R, Lq
    total_entries = sum(entries(o["mesh"].nV, len(o["s"])) for o in objs)
    # device outputs, complex64, one buffer per (object, kind)
    outs = []
    for o, m in zip(objs, meshes):
        nf = len(o["s"])
        per = {}
        for kind in KINDS:
            shape = (nf,) + api.out_shape(L.KINDS[kind], m.nV)
            per[kind] = torch.empty(shape, dtype=torch.complex64, device=dev)
        outs.append(per)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # batched path: every frequency of every object in persistent launches replayed as one CUDA graph
    batch = api.Batch(ctx, KINDS, L.C64)
    for o, m, per in zip(objs, meshes, outs):
        batch.add(m, o["mat"], o["s"], per, order=o["order"], subdiv=o["subdiv"])
    batch.finalize()
    launches_per_step = batch.launches_per_step

    def step():
        batch.run()

    def step_per_object():
        for o, m, per in zip(objs, meshes, outs):
            api.assemble_all(ctx, m, o["mat"], o["s"], order=o["order"], subdiv=o["subdiv"], outs=per, dtype=L.C64)

    def step_plain():
        # the reference's structure: one call per (object, kind, frequency), outputs in device memory
        for o, m, per in zip(objs, meshes, outs):
            for kind in KINDS:
                for l, sl in enumerate(o["s"]):
                    api.assemble(ctx, m, kind, o["mat"], sl, order=o["order"], subdiv=o["subdiv"],
                                 out=per[kind][l], dtype=L.C64)

    def timed(fn, n):
        ts = []
        for _ in range(n):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        return float(sum(ts)) / n

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()  # evict L2 between steps (untimed)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    launches = ctx.launches - launches0
    torch.cuda.synchronize()
    t_max = max_over_ranks(torch, float(sum(times)), dist, dev)
    value = world * total_entries * args.steps / t_max
    # check of the timed step's own outputs (after the timed region): sampled rows against the FP64 oracle
    accuracy = None if args.value_only else check_batched_rows(objs, outs)

    # ---- end to end: the per-object frequency-loop drop-in with pinned host buffers ----
    # Two host threads, each with its own context (stream) and meshes, call sod_cqbem_assemble_all for
    # their share of the objects (largest first, balanced by output bytes), so that one object's compute
    # overlaps the other thread's device-to-host copies; every call returns with its outputs complete in
    # host memory.  Per thread and kind one pinned array of its largest (frequencies x rows x columns)
    # complex128 output, reused by every call as the reference's loops reuse their host matrices.
    e2e_threads = max(1, args.e2e_threads)
    def out_bytes(o, m):
        return sum(len(o["s"]) * int(np.prod(api.out_shape(L.KINDS[k], m.nV))) * 16 for k in KINDS)
    order_ = sorted(range(len(objs)), key=lambda i: -out_bytes(objs[i], meshes[i]))
    shares, load = [[] for _ in range(e2e_threads)], [0] * e2e_threads
    for i in order_:
        t_ = load.index(min(load))
        shares[t_].append(i)
        load[t_] += out_bytes(objs[i], meshes[i])
    workers = []
    for t_ in range(e2e_threads):
        if not shares[t_] or args.no_e2e or args.value_only:
            continue
        wstream = torch.cuda.Stream(dev)
        wctx = ctx if t_ == 0 else api.Context(local, stream=wstream)
        wmeshes = {i: (meshes[i] if t_ == 0 else api.Mesh(wctx, objs[i]["mesh"])) for i in shares[t_]}
        whost = {}
        for kind in KINDS:
            elems = max(len(objs[i]["s"]) * int(np.prod(api.out_shape(L.KINDS[kind], objs[i]["mesh"].nV)))
                        for i in shares[t_])
            whost[kind] = torch.empty(elems, dtype=torch.complex128, pin_memory=True)
        workers.append((wctx, wmeshes, whost, shares[t_]))
    e2e_steps = max(1, args.steps // 2)

    def e2e_worker(w):
        wctx, wmeshes, whost, share = w
        d2h = 0
        for i in share:
            o, m = objs[i], wmeshes[i]
            outs_h = {}
            for kind in KINDS:
                shape = (len(o["s"]),) + tuple(api.out_shape(L.KINDS[kind], m.nV))
                outs_h[kind] = whost[kind][: int(np.prod(shape))].view(shape).numpy()
                d2h += outs_h[kind].nbytes
            api.assemble_all(wctx, m, o["mat"], o["s"], order=o["order"], subdiv=o["subdiv"], outs=outs_h,
                             dtype=L.C128)
        return d2h

    import concurrent.futures as _cf
    e2e_pool = _cf.ThreadPoolExecutor(max(1, len(workers)))

    def e2e_step():
        return sum(e2e_pool.map(e2e_worker, workers))

    e2e_value, d2h_bytes = None, 0
    if not (args.no_e2e or args.value_only):
        for _ in range(2):  # warm the staging buffers, the second context's mesh schedules and the link
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            d2h_bytes = e2e_step()
        torch.cuda.synchronize()
        e2e_t = time.perf_counter() - t0
        e2e_value = world * total_entries * e2e_steps / e2e_t
    e2e_pool.shutdown()
    e2e_nthreads = len(workers)
    for wctx, wmeshes, whost, share in workers:
        if wctx is ctx:
            continue
        for m_ in wmeshes.values():
            m_.close()
        wctx.close()
    del workers
    # ---- the same workload through the per-object and the plain per-(kind, frequency) drop-in ----
    t_per_object = t_plain = None
    if not args.value_only:
        step_per_object()
        step_plain()
        torch.cuda.synchronize()
        t_per_object = timed(step_per_object, max(1, args.steps // 2))
        t_plain = timed(step_plain, max(1, args.steps // 2))

    h2d_bytes = sum(16 * len(o["s"]) + 64 for o in objs)  # per-call frequency constants

    # ---- roofline of the dominant kernel of the batched step: per-launch CUDA-event times ----
    peak_fp32 = measure_fp32_peak(torch, dev)
    prof = batch.profile()
    for _ in range(2):
        p2 = batch.profile()
        for a_, b_ in zip(prof, p2):
            a_["ms"] = min(a_["ms"], b_["ms"])
    step_ms = sum(p["ms"] for p in prof)
    fp32 = [p for p in prof if p["pass"] in PASS_FLOPS]
    dom = max(fp32, key=lambda p: p["ms"])
    achieved = dom["evals"] * PASS_FLOPS[dom["pass"]] / (dom["ms"] * 1e-3) / 1e12
    traffic = TRAFFIC_BYTES_PER_EVAL.get(dom["pass"])
    names = {"scatter_G": "batch_scatter_kernel<G, B_trans|B_angular>", "scatter_H": "batch_scatter_kernel<H>",
             "reduce_B": "batch_reduce_kernel<B_trans|B_angular>"}
    roofline = {"bound": "fp32", "kernel": names[dom["pass"]],
                "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s", "frac": achieved / peak_fp32,
                "peak_source": "measured live: cuBLAS SGEMM 8192^3, TF32 off (no FP32 figure in the measured "
                               "peaks file)",
                "traffic": traffic * dom["evals"] if traffic else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per evaluation, scaled by "
                                  "the launch's evaluations" if traffic else None,
                "flops_per_eval": PASS_FLOPS[dom["pass"]], "evals_per_launch": dom["evals"],
                "launch_ms": dom["ms"], "launch_share": dom["ms"] / step_ms,
                "launches": [{"pass": p["pass"], "ms": round(p["ms"], 3), "share": round(p["ms"] / step_ms, 4),
                              "evals": p["evals"]} for p in prof]}

    # ---- other hot-path legs: history convolution, elastostatics, the request loop ----
    extra = {}
    if not args.value_only and args.case == "mixed24":
        del outs, batch
        torch.cuda.empty_cache()
        extra["history_convolution"] = history_leg(torch, ctx, stream)
        extra["precompute"] = precompute_leg(torch, ctx, stream)
        extra["elastostatic"] = elastostatic_leg(torch, ctx, stream)
        extra["galerkin"] = galerkin_leg(torch, ctx, stream)
        extra["dense_solve"] = solve_leg(torch, ctx, stream)
        extra["reference_scenes"] = scenes_leg(torch, ctx, stream)
        if not args.no_serve:
            extra["serving"] = serving_leg(torch, ctx, n_requests=args.serve_requests, rate_hz=args.serve_rate)

    # ---- CPU baseline (rank 0, N = 1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not (args.no_cpu or args.value_only):
        r, dtc, cores, sample, est = cpu_sample(objs, os.cpu_count() or 1)
        cpu = {"value": r, "unit": "entries/s", "cores": cores, "kind": "port", "sample": sample,
               "seconds": dtc, "estimated_step_s": est}
    paths = {"batched_graph": {"entries_per_s": value, "launches_per_step": launches_per_step}}
    if t_plain:
        paths["per_object_fused"] = {"entries_per_s": total_entries / t_per_object, "ms_per_step": t_per_object * 1e3}
        paths["plain_per_kind_frequency"] = {"entries_per_s": total_entries / t_plain, "ms_per_step": t_plain * 1e3}
        paths["batched_over_plain"] = t_plain / (t_max / args.steps)
    if rank == 0:
        line = {"metric": "CQBEM Laplace-domain entries/s (mixed-size 24-object set)", "value": value,
                "unit": "entries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32+double-float", "data": "synthetic",
                "config": {"workload": "mixed-size 24-object collocation assembly (G,H,B_trans,B_angular, all "
                                       "Laplace frequencies); batched persistent kernels under one CUDA graph",
                           "objects": len(objs),
                           "vertices": [m.nV for m in meshes], "frequencies": [len(o["s"]) for o in objs],
                           "entries_per_step": total_entries, "quadrature": "7-point (order 5), singular 5x5 FP64",
                           "l2": "L2 flushed (256 MB write) between timed steps; outputs (~"
                                 f"{total_entries * 8 / 1e9:.0f} GB complex64) exceed L2",
                           "parallelism": f"replicas x{world}"},
                "roofline": roofline, "cpu_baseline": cpu, "accuracy": accuracy,
                "paths": paths,
                "batched_over_plain": paths.get("batched_over_plain"),
                "e2e": {"value": e2e_value, "unit": "entries/s", "h2d_bytes_per_step": h2d_bytes,
                        "d2h_bytes_per_step": d2h_bytes, "path": "sod_cqbem_assemble_all per object (the frequency-loop "
                        "drop-in of all four kinds) into pinned host memory, complex128 reference layout, "
                        f"from {e2e_nthreads} host thread(s) with a context each",
                        "steps": e2e_steps},
                "gpu_launches": int(launches), "clocks": clk.summary(), **extra}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def run_leg(args):
    """One hot-path leg on its own, e.g. a smaller history bank for an ncu capture."""
    import torch

    from surfaceonlydeformables_gb300 import api
    from surfaceonlydeformables_gb300 import build as B

    B.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = api.Context(0, stream=stream)
    if args.leg == "history":
        out = history_leg(torch, ctx, stream, K=args.history_k, reps=args.steps)
    elif args.leg == "elastostatic":
        out = elastostatic_leg(torch, ctx, stream)
    elif args.leg == "precompute":
        out = precompute_leg(torch, ctx, stream, levels=(args.precompute_level,))
    elif args.leg == "galerkin":
        out = galerkin_leg(torch, ctx, stream, level=args.galerkin_level)
    elif args.leg == "solve":
        out = solve_leg(torch, ctx, stream, n=args.solve_n)
    elif args.leg == "scenes":
        out = scenes_leg(torch, ctx, stream)
    elif args.leg == "wavelet":
        out = wavelet_case(torch, ctx, stream, args.wavelet_nv, args.history_k, 0.1, args.steps, measured_hbm_gbs())
    else:
        out = serving_leg(torch, ctx, n_requests=args.serve_requests, rate_hz=args.serve_rate)
    print(json.dumps({"leg": args.leg, **out}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop leg")
    ap.add_argument("--e2e-threads", type=int, default=2, help="host threads (one context each) of the e2e leg")
    ap.add_argument("--leg", default="all", choices=["all", "history", "elastostatic", "galerkin", "serving", "solve", "wavelet", "scenes",
                                                     "precompute"],
                    help="run one hot-path leg alone (profiling captures) and print its JSON")
    ap.add_argument("--history-k", type=int, default=64, help="history length of the --leg history bank")
    ap.add_argument("--wavelet-nv", type=int, default=2562,
                    help="vertices of the --leg wavelet compressed bank (642 = the small profiling case)")
    ap.add_argument("--serve-requests", type=int, default=240, help="requests of the serving leg")
    ap.add_argument("--serve-rate", type=float, default=30.0, help="Poisson arrival rate of the serving leg (req/s)")
    ap.add_argument("--solve-n", type=int, default=7686,
                    help="matrix size of the --leg solve systems (1926: the small profiling case)")
    ap.add_argument("--precompute-level", type=int, default=3, choices=[2, 3, 4],
                    help="icosphere level of the --leg precompute object (2: the small profiling case)")
    ap.add_argument("--galerkin-level", type=int, default=4, choices=[3, 4],
                    help="icosphere level of the --leg galerkin mesh (3: the small profiling case)")
    ap.add_argument("--value-only", action="store_true",
                    help="profiling runs: time the batched step only (no comparison paths, e2e or CPU leg)")
    ap.add_argument("--case", default="mixed24", choices=sorted(CASES),
                    help="workload: the 24-object set (default) or one object for profiling captures")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.leg != "all":
        return run_leg(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
