"""Benchmark: single-graph truss decomposition on one GB300 (edges/s).

Workload (N=1): R-MAT scale 22, edge factor 16 (2^26 draws),
(a,b,c,d) = (0.57, 0.19, 0.19, 0.05), seed 1, symmetrised, deduplicated and
degree-oriented (int32 CSR, int64 row offsets).  A step = one full
decomposition (support pass + every peel level + the e_truss/ptr_truss
outputs) of that graph.

* value: edges/s with the CSR resident in HBM (inputs larger than L2);
* e2e:   the same through truss_decompose with host buffers: each step
         copies the CSR (columns, row_ptr) from pinned host memory (the COO
         rows are derived on the device) and reads the per-edge truss
         numbers back;
* roofline: algorithmic bytes over CUDA-event time: a decomposition moves
         B_dec = 2 B_sup (B_sup = 4W + 28E + 4(V+1), W = sum over edges of
         d+(u)+d+(v)): the support pass, then one re-enumeration of each
         edge's triangles (listing + peel); DRAM traffic per decomposition
         from one ncu capture of this workload sits beside it;
* cpu_baseline: the oracle port of the reference's CPU flow (OpenMP, all host
         cores) on a bounded R-MAT sample.

--impl reference times the reference's CPU implementation (the oracle port,
all host threads) on the same metric.  Multi-GPU (torchrun): replicas only;
each rank decomposes its own copy, value = ranks * E / max step time.
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

METRIC = "edges/s decomposed"
UNIT = "edges/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--lists", choices=["auto", "on", "off"], default="auto",
                    help="triangle lists of the main decomposition: auto (whenever they fit), on, or off (the search "
                         "peel, as on graphs whose lists do not fit)")
    ap.add_argument("--cpu-scale", type=int, default=0, help="R-MAT scale of the CPU sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-skewed", action="store_true", help="skip the Chung-Lu 2^25 section")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own GPU kernels beside this build's")
    ap.add_argument("--no-same-scale", action="store_true",
                    help="skip the GPU decomposition of the CPU arm's graph")
    ap.add_argument("--skewed", action="store_true",
                    help="also run the skewed Chung-Lu graph (n=2^25): triangle count, decomposition, k-truss")
    ap.add_argument("--skewed-log2n", type=int, default=25)
    ap.add_argument("--fusion", action="store_true",
                    help="add the fusion-experiment line (unfused vs fused support count)")
    ap.add_argument("--fusion-scale", type=int, default=18)
    ap.add_argument("--undirected", action="store_true",
                    help="add the undirected-driver line (oriented and symmetric peel updates)")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    import torch.distributed as dist
    if ws > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend)
    return dist


def max_over_ranks(x, ws, device):
    import torch
    import torch.distributed as dist
    if ws == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    import torch.distributed as dist
    if ws > 1:
        dist.barrier()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU legs (oracle)
def cpu_sample_scale(args, steps):
    """R-MAT scale of the CPU arm for a run of `steps` decompositions (warm-up
    included): the same in the reference arm, the cpu_baseline leg and the
    GPU line's same_scale object of a run with the same --steps/--warmup
    (about 10-40 s of host work on the box's 16 cores)."""
    if args.cpu_scale:
        return args.cpu_scale
    return 18 if steps <= 4 else (17 if steps <= 15 else (16 if steps <= 40 else 15))


def cpu_decompose_sample(scale, reps, warm=0):
    """The oracle port of the reference's `--cuda` flow (singlegpu_truss.py
    k_truss, OpenMP ops) on R-MAT(scale, 16*2^scale draws, seed 1).  Returns
    (E, V, seconds per run, threads, per-edge truss numbers of the last run)."""
    import numpy as np
    from oracle import oracle as O
    from tdtdecomposition_gb300 import generators as G
    s, d = G.rmat_edges(scale, 16 << scale, seed=1)
    rows, cols, rp, verts = O.preprocess(np.stack([s, d], 1))
    V = len(verts)
    rpt = O.tiling_row_ptr(rows, cols, V, 2)
    for _ in range(warm):
        O.k_truss(rows, cols, rpt, V, 2)
    times = []
    truss = None
    for _ in range(reps):
        t = time.perf_counter()
        truss = O.k_truss(rows, cols, rpt, V, 2)[3]
        times.append(time.perf_counter() - t)
    return len(cols), V, times, O.num_threads(), truss


def reference_arm(args):
    ws, rank, _ = dist_env()
    if ws > 1:
        dist_init(ws, "gloo")
        if rank != 0:
            return
    scale = cpu_sample_scale(args, args.steps + args.warmup)
    E, V, times, threads, _ = cpu_decompose_sample(scale, args.steps, args.warmup)
    t = sum(times)
    value = E * len(times) / t
    sample = "R-MAT scale %d, 16*2^%d draws, seed 1 (V=%d, E=%d), one full decomposition per step" % (
        scale, scale, V, E)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic",
            "config": {"workload": "R-MAT single-graph truss decomposition (CPU sample of scale %d)" % scale,
                       "scale": scale, "edge_factor": 16, "V": V, "E": E},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- batched workload
def bench_batched(dev, steps, warmup, num_graphs=4096):
    """4096 Barabasi-Albert graphs (n log-uniform in [64, 16384], m uniform in
    {4..16}, graph i seeded 1000+i): one device-resident run over their
    disjoint union vs the plain path (one truss_decompose call per graph)."""
    import torch
    from tdtdecomposition_gb300 import autotune, batch as B, graph as GR, serve as S, truss as T, workloads as W
    from tdtdecomposition_gb300.preprocess import group_offsets, preprocess_edges
    t0 = time.perf_counter()
    src, dst, vg = W.ba_batch_edges(num_graphs, seed=1000)
    t_gen = time.perf_counter() - t0
    vg_d = torch.as_tensor(vg).to(dev)
    g, verts = preprocess_edges(torch.as_tensor(src).to(dev), torch.as_tensor(dst).to(dev), vg_d)
    vo, eo = group_offsets(vg_d, verts, g)
    bt = B.batch_from_union(g, eo, vo)
    E = g.num_edges
    wsb = T.Workspace(dev)
    tuned = autotune.tune(g, workspace=wsb)  # (warp_cap, heavy_cap, lists, peel_grid, vec)
    for _ in range(warmup):
        B.decompose(bt, workspace=wsb, lists=tuned[2], sync=False)
    torch.cuda.synchronize()
    ref = B.decompose(bt, workspace=wsb, lists=tuned[2])
    stream = torch.cuda.current_stream(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        B.decompose(bt, workspace=wsb, lists=tuned[2], sync=False)
    b.record(stream)
    torch.cuda.synchronize()
    ms_batched = a.elapsed_time(b) / steps
    # the same run recorded once as a CUDA graph and replayed
    cap = B.capture(bt, workspace=T.Workspace(dev), lists=tuned[2])
    for _ in range(warmup):
        cap.replay(sync=False)
    torch.cuda.synchronize()
    rep = cap.replay()
    if not torch.equal(rep.truss, ref.truss):
        raise SystemExit("CUDA-graph replay differs from the eager batched run")
    a.record(stream)
    for _ in range(steps):
        cap.replay(sync=False)
    b.record(stream)
    torch.cuda.synchronize()
    ms_graph = a.elapsed_time(b) / steps
    del cap
    autotune.reset()
    # plain path: the same graphs, one call (and one result read-back) per graph
    eoh, voh = eo.cpu().tolist(), vo.cpu().tolist()
    singles = []
    for i in range(num_graphs):
        ea, eb_, va, vb_ = eoh[i], eoh[i + 1], voh[i], voh[i + 1]
        singles.append(GR.CSRCOO(columns=g.columns[ea:eb_] - va, row_ptr=g.row_ptr[va:vb_ + 1] - ea,
                                 rows=g.rows[ea:eb_] - va))
    # (the list decision made on the device, as the server makes it: lists
    # when 24 T bytes fit the tail, no counting pass per graph)
    wsp = T.Workspace(dev)
    for sg in singles[:8]:
        T.truss_decompose(sg, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    outs = [T.truss_decompose(sg, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET).truss for sg in singles]
    torch.cuda.synchronize()
    s_plain = time.perf_counter() - t1
    same = all(torch.equal(o, ref.truss[eoh[i]:eoh[i + 1]]) for i, o in enumerate(outs))
    if not same:
        raise SystemExit("batched result differs from the per-graph results")
    return {"workload": "4096 Barabasi-Albert graphs, n log-uniform [64,16384], m uniform {4..16}, seeds 1000+i",
            "graphs": num_graphs, "V": int(g.num_vertices), "E": int(E),
            "value": E / (ms_batched / 1e3), "unit": UNIT, "ms_per_step": ms_batched,
            "plain_value": E / s_plain, "plain_s": s_plain, "speedup_vs_plain": (E / (ms_batched / 1e3)) / (E / s_plain),
            "kmax_max": int(ref.kmax.max()), "sub_rounds": ref.union.rounds,
            "cuda_graph": {"ms_per_step": ms_graph, "value": E / (ms_graph / 1e3),
                           "note": "support, listing, the cooperative peel and outputs captured once, replayed"},
            "autotuned": {"warp_cap": tuned[0], "heavy_cap": tuned[1], "lists": tuned[2],
                          "peel_grid_half_sms": tuned[3], "vector_walk": tuned[4]},
            "host_generation_s": t_gen, "results_identical_to_plain": True}


# ---------------------------------------------------------------- skewed single graph
def bench_skewed(dev, log2n=25):
    """Chung-Lu power law (exponent 2.1, n = 2^log2n, mean degree 40, degree
    cap 2^20, seed 2), generated, deduplicated and degree-oriented on the
    GPU; triangle count, full decomposition (per-edge triangle lists when 24 T
    bytes fit the device, else the search peel) and k-truss search at
    k in {3, 8, kmax/2, kmax}, each checked against {e : truss(e) >= k}.
    One run each (seconds to a minute)."""
    import torch
    from tdtdecomposition_gb300 import generators as G, truss as T
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    n = 1 << log2n
    peak = _hbm_peak()[0]

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t

    (s, d), t_gen = timed(lambda: G.chung_lu_edges_device(n, seed=2, device=dev))
    draws = s.numel()
    (g, _), t_pre = timed(lambda: preprocess_edges(s, d))
    del s, d
    E, V = g.num_edges, g.num_vertices
    ws = T.Workspace(dev)
    T.triangle_count(g, workspace=ws)
    tri, t_tc = timed(lambda: T.triangle_count(g, workspace=ws))
    res, t_dec = timed(lambda: T.truss_decompose(g, workspace=ws))
    truss = res.truss
    # algorithmic bytes: B_sup = 4 W + 28 E + 4 (V+1); decomposition 2 B_sup;
    # k-truss search B_sup + 4 W_del + 28 E, W_del = W over the deleted edges
    rp = g.row_ptr.to(torch.int64)
    dplus = rp[1:] - rp[:-1]
    rows = g.rows if g.rows is not None else torch.repeat_interleave(torch.arange(V, device=dev), dplus)
    wpe = dplus[rows.long()] + dplus[g.columns.long()]
    W = int(wpe.sum())
    B_sup = 4 * W + 28 * E + 4 * (V + 1)

    def roof(B, t):
        return {"algorithmic_bytes": B, "achieved_gbs": B / t / 1e9, "frac": B / t / 1e9 / peak}

    kt = {}
    for k in sorted({3, 8, res.kmax // 2, res.kmax}):
        m, tk = timed(lambda: T.ktruss_search(g, k, workspace=ws))
        if not torch.equal(m, truss >= k):
            raise SystemExit("k-truss at k=%d differs from {e : truss(e) >= k}" % k)
        W_del = int(wpe[~m].sum())
        kt[str(k)] = dict({"edges": int(m.sum()), "s": tk, "edges_per_s": E / tk},
                          **roof(B_sup + 4 * W_del + 28 * E, tk))
    return {"workload": "Chung-Lu n=2^%d, exponent 2.1, mean degree 40, degree cap 2^20, seed 2" % log2n,
            "draws": draws, "V": V, "E": E, "W": W, "triangles": tri, "kmax": res.kmax, "rounds": res.rounds,
            "generate_s": t_gen, "preprocess_s": t_pre, "preprocess_draws_per_s": draws / t_pre,
            "triangle_count_s": t_tc, "triangle_count_edges_per_s": E / t_tc,
            "triangle_count_roofline": roof(B_sup, t_tc),
            "decompose_s": t_dec, "value": E / t_dec, "unit": UNIT, "decompose_roofline": roof(2 * B_sup, t_dec),
            "peak_gbs": peak,
            "peel_mode": {2: "lists (one walk)", 1: "lists (two walks)"}.get(
                res.listing, "search (24 T bytes of lists exceed the device budget)"),
            "ktruss": kt, "ktruss_equals_truss_ge_k": True}


def _hbm_peak():
    """(GB/s, 'measured' | 'fallback'): the copy bandwidth the pool measured on
    this GPU model, else the fallback figure."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


# ---------------------------------------------------------------- reference GPU path
def bench_reference_gpu(dev, g, ws, flow_scale=18, reps=3):
    """The reference's own GPU kernels (myhpu_extension_kernel.cu compiled
    unmodified for sm_103a; oracle/ref_gpu.py launches them as the
    reference's launchers do) beside this build's, on the same GPU:

    * support pass on the benchmark graph: checkElementsTwoPtrTile (K3,
      kernel.cu:81-141, n_cut = 2) against the build's count walk
      (tdt_triangle_count), CUDA events, same per-edge support required;
    * the reference's `--cuda` flow (singlegpu_truss.py:67-158, restated in
      flow.k_truss, its torch glue unchanged) over the reference's kernels
      (K3, AllAffectedSupport_tilenot K7, segmentAdd K1) against
      truss_decompose, on R-MAT(flow_scale), same e_truss / ptr_truss
      required."""
    import torch
    try:
        from oracle import ref_gpu as RG
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "oracle/ref_gpu.py not importable: %s" % e}
    if not RG.available():
        return {"unavailable": "reference kernel image not built (oracle/build.py compiles it where the "
                               "reference tree is present)"}
    from tdtdecomposition_gb300 import CSRCOO, generators as G, truss as T
    from tdtdecomposition_gb300.graph import tiling_row_ptr
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    K = RG.RefKernels()
    stream = torch.cuda.current_stream(dev)

    def ev_time(fn, n):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    rows = g.rows if g.rows is not None else torch.repeat_interleave(
        torch.arange(g.num_vertices, device=dev, dtype=torch.int32), g.row_ptr[1:] - g.row_ptr[:-1])
    rpt = tiling_row_ptr(CSRCOO(columns=g.columns, row_ptr=g.row_ptr, rows=rows), 2)
    out = torch.zeros(g.num_edges, dtype=torch.int32, device=dev)

    def ref_support():
        out.zero_()
        K.segment_isin2tile(rows, g.columns, rpt, 2, out)

    t_ref = ev_time(ref_support, reps)
    _, sup = T.triangle_count(g, workspace=ws, return_support=True)
    same = bool(torch.equal(out, sup))
    t_ours = ev_time(lambda: T.triangle_count(g, workspace=ws), reps)
    del out, rpt, sup
    # the host-driven flow over the reference's kernels, R-MAT(flow_scale)
    src, dst = G.rmat_edges_device(flow_scale, 16 << flow_scale, seed=1, device=dev)
    h, verts = preprocess_edges(src, dst)
    del src, dst
    V, E = h.num_vertices, h.num_edges
    wsf = T.Workspace(dev)
    mine = T.truss_decompose(h, workspace=wsf)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mine = T.truss_decompose(h, workspace=wsf)
    t_mine = time.perf_counter() - t0

    def ref_flow():
        gg = CSRCOO(columns=h.columns.clone(), row_ptr=tiling_row_ptr(h, 2), rows=h.rows.clone())
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = RG.k_truss_on_reference_kernels(gg, 2, V, K)
        torch.cuda.synchronize()
        return res, time.perf_counter() - t

    ref_flow()  # warm-up (module, allocator)
    (kmax, et, pt), t_flow = ref_flow()
    ident = (kmax == mine.kmax and torch.equal(et.to(dev), mine.e_truss)
             and torch.equal(pt.cpu(), mine.ptr_truss.cpu()))
    if not (same and ident):
        print(json.dumps({"error": "reference GPU kernels disagree with the build", "support_equal": same,
                          "flow_equal": ident}), file=sys.stderr, flush=True)
    return {"image": "myhpu_extension_kernel.cu compiled unmodified for sm_103a",
            "support_pass": {"workload": "the benchmark graph (E=%d), n_cut = 2" % g.num_edges,
                             "reference_kernel": "checkElementsTwoPtrTile (K3)", "reference_ms": t_ref,
                             "ours_kernel": "support_kernel (count walk, tdt_triangle_count)", "ours_ms": t_ours,
                             "speedup": t_ref / t_ours, "same_support": same},
            "flow": {"workload": "R-MAT scale %d, edge factor 16, seed 1 (V=%d, E=%d)" % (flow_scale, V, E),
                     "reference": "singlegpu_truss.k_truss flow over the reference kernels (n_cut = 2)",
                     "reference_s": t_flow, "reference_edges_per_s": E / t_flow,
                     "ours": "truss_decompose", "ours_s": t_mine, "ours_edges_per_s": E / t_mine,
                     "speedup": t_flow / t_mine, "results_identical": bool(ident)},
            "reference_kernel_launches": K.launches}


def bench_same_scale(dev, scale, reps):
    """The GPU decomposition of exactly the graph the CPU arm times: R-MAT
    (scale, 16 * 2^scale draws, seed 1), generated and preprocessed on the
    device (the same edges and CSR as the oracle's).  Returns the line and
    the per-edge truss numbers for the comparison with the CPU result."""
    import torch
    from tdtdecomposition_gb300 import generators as G, truss as T
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    src, dst = G.rmat_edges_device(scale, 16 << scale, seed=1, device=dev)
    g, _ = preprocess_edges(src, dst)
    del src, dst
    ws = T.Workspace(dev)
    for _ in range(2):
        T.truss_decompose(g, workspace=ws)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        res = T.truss_decompose(g, workspace=ws, sync=False)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    truss = res[0].cpu().numpy()
    return {"scale": scale, "V": g.num_vertices, "E": g.num_edges, "gpu_ms": ms,
            "gpu_value": g.num_edges / (ms / 1e3), "unit": UNIT}, truss


# ---------------------------------------------------------------- fusion ablation
def bench_fusion(dev, scale=18, reps=3):
    """The fusion experiment (fusionexperiental.py:24-46, EXP3 "ComputeSup"
    vs "ComputeSup+") on R-MAT scale `scale`, edge factor 16, seed 1: the
    unfused support count (gather both out-lists of every edge,
    segment_isinmm, segment_add and two unique/count passes) against the
    fused segment_isin2 drop-in op.  Both give the same supports (checked).
    Median of `reps` timed runs after one warm-up each."""
    import torch
    from tdtdecomposition_gb300 import flow, generators as G
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    src, dst = G.rmat_edges_device(scale, 16 << scale, seed=1, device=dev)
    g, _ = preprocess_edges(src, dst)
    del src, dst
    rp32 = g.row_ptr.to(torch.int32)
    deg = (g.row_ptr[1:] - g.row_ptr[:-1])
    gathered = int(deg[g.rows.long()].sum()) + int(deg[g.columns.long()].sum())
    free, _ = torch.cuda.mem_get_info(dev)
    if gathered * 24 > 0.6 * free:
        return {"workload": "R-MAT scale %d, edge factor 16, seed 1" % scale,
                "skipped": "the unfused count gathers %d list entries; too large for free memory" % gathered}

    def timed(fn):
        fn()
        out, ms = None, []
        for _ in range(reps):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            out = fn()
            b.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return out, sorted(ms)[len(ms) // 2]

    fused, t_fused = timed(lambda: flow.support_computing(g.rows, g.columns, rp32, 1))
    unfused, t_unfused = timed(lambda: flow.support_computing_before(g.rows, g.columns, rp32, 1))
    if not torch.equal(fused, unfused):
        raise SystemExit("unfused and fused support counts differ")
    out = {"workload": "R-MAT scale %d, edge factor 16, seed 1" % scale, "V": g.num_vertices, "E": g.num_edges,
           "gathered_list_entries": gathered, "triangles": int(fused.to(torch.int64).sum()) // 3,
           "compute_sup_ms": t_unfused, "compute_sup_plus_ms": t_fused, "fused_speedup": t_unfused / t_fused}
    # the full-decomposition ablation (EXP3.2 columns) on the reference's
    # host-driven flow (n_cut = 1), and the device-resident path beside it
    from tdtdecomposition_gb300 import CSRCOO, truss as T
    abl, want = {}, None
    for name, fs, fu in (("TDT-origin", False, False), ("+Comp", True, False), ("+Update", False, True),
                         ("+both", True, True)):
        h = CSRCOO(columns=g.columns.clone(), row_ptr=rp32.clone(), rows=g.rows.clone())
        torch.cuda.synchronize()
        t = time.perf_counter()
        kmax, et, pt = flow.k_truss(h, 1, g.num_vertices, fused_support=fs, fused_update=fu)
        torch.cuda.synchronize()
        abl[name] = time.perf_counter() - t
        if want is None:
            want = (kmax, et, pt)
        elif kmax != want[0] or not torch.equal(et, want[1]) or not torch.equal(pt, want[2]):
            raise SystemExit("ablation variant %s peels differently" % name)
    res = T.truss_decompose(g)
    torch.cuda.synchronize()
    t = time.perf_counter()
    res = T.truss_decompose(g)
    abl["device-resident"] = time.perf_counter() - t
    if res.kmax != want[0] or not torch.equal(res.e_truss.to(torch.int32), want[1].to(torch.int32)):
        raise SystemExit("the device-resident decomposition peels differently from the flow")
    out["decomposition_s"] = abl
    out["kmax"] = want[0]
    return out


# ---------------------------------------------------------------- undirected drivers
def bench_undirected(dev, scale=18):
    """The reference's undirected-graph drivers (truss_undirect_cuda2.py with
    the oriented peel updates, truss_undirect_cuda.py with the symmetric one)
    restated over this library's operators, on R-MAT scale `scale`, edge
    factor 16, seed 1, n_cut 1; one run each after a warm-up, checked against
    the device-resident decomposition (same kmax, same per-edge truss)."""
    import torch
    from tdtdecomposition_gb300 import flow, generators as G, truss as T
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    src, dst = G.rmat_edges_device(scale, 16 << scale, seed=1, device=dev)
    g, _ = preprocess_edges(src, dst)
    del src, dst
    res = T.truss_decompose(g)
    E = g.num_edges

    def truss_of(e, p):
        t = torch.full((E,), 2, dtype=torch.int32, device=dev)
        lv = torch.repeat_interleave(torch.arange(p.numel() - 1, device=dev, dtype=torch.int32) + 3,
                                     (p[1:] - p[:-1]).to(dev).long())
        t[e.long()] = lv
        return t

    out = {"workload": "R-MAT scale %d, edge factor 16, seed 1" % scale, "E": E, "kmax": res.kmax}
    runs = (("oriented (peeling_direct_oo/ii/oi)",
             lambda: flow.undirected_truss_direct(g, *flow.preprocess_direct(g, 1), 1)),
            ("symmetric (peeling_undirect)",
             lambda: (lambda parts: flow.undirected_truss_undirect(g, parts[1], parts[2], parts[0], parts[3], 1, 1))(
                 flow.preprocess_undirect(g, 1, 1))))
    for name, fn in runs:
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        k, e, p = fn()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        if k != res.kmax or not torch.equal(truss_of(e, p), res.truss):
            raise SystemExit("undirected driver %s differs from the decomposition" % name)
        out[name] = {"s": dt, "edges_per_s": E / dt}
    torch.cuda.synchronize()
    t = time.perf_counter()
    T.truss_decompose(g)
    torch.cuda.synchronize()
    out["device-resident s"] = time.perf_counter() - t
    return out


# ---------------------------------------------------------------- served workload
def bench_served(dev, n_requests=1000, rates=(64.0, 256.0, 1024.0), n_resident=200):
    """Poisson request streams (the same n_requests seeded requests replayed
    at each rate): half Barabasi-Albert (n log-uniform [256, 2^18], m in
    {4..16}), half R-MAT (scale 12..20, edge factor 16); half full
    decompositions, half k-truss searches (k uniform in [3, 20]); 150 GB
    admission budget.  The plain path serves the same requests one at a time
    with the same per-request choice (copy in, preprocess, decompose -- or
    the fixed-level search for a k-truss query on a graph of 2^19 edges or
    more -- answer out).  Then n_resident follow-up queries (a k-truss at
    another k, a decomposition, a triangle count) on graphs the last stream
    kept resident, answered without ingest."""
    import numpy as np
    import torch
    from tdtdecomposition_gb300 import serve as S, truss as T, workloads as W
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    specs = W.request_stream(n_requests, rate_per_s=1.0, seed=7)
    base = S.make_requests(specs, device=dev)
    draws = sum(len(r.src) for r in base)
    search_min = 1 << 19
    wsp, pps = T.Workspace(dev), T.Workspace(dev)
    big = max(base, key=lambda r: len(r.src))  # grows both workspaces before the timed loop
    gb, _ = preprocess_edges(big.src.to(dev), big.dst.to(dev), workspace=pps)
    T.truss_decompose(gb, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET)
    del gb
    plain_answers, edges, sizes = [], 0, []
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for r in base:
        g, _ = preprocess_edges(r.src.to(dev, non_blocking=True), r.dst.to(dev, non_blocking=True), workspace=pps)
        edges += g.num_edges
        sizes.append(g.num_edges)
        if S.is_ktruss(r.query) and g.num_edges >= search_min:
            a = T.ktruss_search(g, int(r.query[1]), workspace=wsp, lists=False)
        else:
            a = S.answer_for(r.query, T.truss_decompose(g, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET).truss)
        plain_answers.append(a.cpu())
    s_plain = time.perf_counter() - t1
    del wsp, pps
    torch.cuda.empty_cache()
    out = {"workload": "Poisson stream of %d requests: half BA n log-uniform [256,2^18] m {4..16}, half R-MAT "
                       "scale 12..20 ef 16; half decompose, half k-truss k in [3,20]; 150 GB budget" % n_requests,
           "requests": n_requests, "edges": edges, "draws": draws,
           "requests_by_class": {name: int(sum(lo <= e < hi for e in sizes)) for name, lo, hi in S.SIZE_CLASSES},
           "plain_value": edges / s_plain, "plain_s": s_plain,
           "plain": "one request at a time: copy in, preprocess, decompose (or the fixed-level search for a "
                    "k-truss query on >= 2^19 edges), answer out",
           "server": {"max_batch_edges": 1 << 23, "max_wait_s": 0.25, "search_min_edges": search_min}, "rates": []}
    srv = S.TrussServer(dev, memory_budget=150e9, search_min_edges=search_min)
    srv.run([S.Request(r.id, 0.0, r.src, r.dst, r.query) for r in base[:8]], real_time=False)  # warm-up
    reqs = None
    for lam in rates:
        keep_last = lam == rates[-1]
        reqs = [S.Request(r.id, sp["arrival"] / lam, r.src, r.dst, r.query, handle=r.id,
                          keep=keep_last and r.id % (n_requests // n_resident) == 0)
                for r, sp in zip(base, specs)]
        srv.run(reqs, real_time=True)
        for r, a in zip(reqs, plain_answers):
            if not torch.equal(r.answer, a):
                raise SystemExit("served answer of request %d differs from the request run alone" % r.id)
        st = S.latency_stats(reqs)
        span = max(r.t_done for r in reqs) - min(r.arrival for r in reqs)
        out["rates"].append({"rate_per_s": lam, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                             "value": edges / span, "unit": UNIT, "makespan_s": span,
                             "by_class": S.latency_by_class(reqs),
                             "paths": {p: sum(r.path == p for r in reqs) for p in ("batch", "search")}})
    best = max(out["rates"], key=lambda x: x["value"])
    out["value"] = best["value"]
    out["unit"] = UNIT
    out["speedup_vs_plain"] = best["value"] / out["plain_value"]
    out["results_identical_to_plain"] = True
    # follow-up queries on the graphs the last stream kept resident
    kept = [r for r in reqs if r.keep]
    rng = np.random.default_rng(3)
    follow = []
    for i, r in enumerate(kept):
        q = ("ktruss", int(rng.integers(3, 21))) if i % 3 == 0 else ("decompose" if i % 3 == 1 else "triangles")
        follow.append(S.Request(n_requests + i, 0.005 * i, None, None, q, handle=r.handle))
    srv.run(follow, real_time=True)  # one query every 5 ms
    checked = 0
    for q, r in zip(follow, kept):
        if q.query == "decompose":
            ok = torch.equal(q.answer, plain_answers[r.id]) if r.query == "decompose" else True
            checked += r.query == "decompose"
            if not ok:
                raise SystemExit("resident decomposition of request %d differs" % r.id)
    st = S.latency_stats(follow)
    out["resident_followups"] = {"queries": len(follow), "arrivals": "one every 5 ms",
                                 "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                                 "resident_graphs": len(srv.resident), "resident_bytes": srv.resident_bytes,
                                 "decompositions_checked_against_plain": checked}
    out["small_graphs"] = bench_served_small(dev, srv)
    return out


def bench_served_small(dev, srv, num_graphs=4096, rate=20000.0):
    """The many-small-graph workload of the batched section (4096 BA graphs)
    as a request stream (Poisson, 20000 requests/s, alternating full
    decompositions and k-truss searches with k in [3, 20]) through the
    server, against the plain path that serves the same requests one at a
    time (copy in, preprocess, decompose, answer out)."""
    import numpy as np
    import torch
    from tdtdecomposition_gb300 import generators as G, serve as S, truss as T, workloads as W
    from tdtdecomposition_gb300.preprocess import preprocess_edges
    n, m = W.ba_batch_params(num_graphs, seed=1000)
    rng = np.random.default_rng(17)
    t = np.cumsum(rng.exponential(1.0 / rate, num_graphs))
    base = []
    for i in range(num_graphs):
        s_, d_ = G.ba_edges(int(n[i]), int(m[i]), 1000 + i)
        q = "decompose" if i % 2 == 0 else ("ktruss", int(rng.integers(3, 21)))
        base.append(S.Request(i, float(t[i]), torch.from_numpy(s_).pin_memory(), torch.from_numpy(d_).pin_memory(), q))
    wsp, pps = T.Workspace(dev), T.Workspace(dev)
    big = max(base, key=lambda r: len(r.src))  # grows both workspaces before the timed loop
    gb, _ = preprocess_edges(big.src.to(dev), big.dst.to(dev), workspace=pps)
    T.truss_decompose(gb, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET)
    del gb
    plain_answers, edges = [], 0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for r in base:
        g, _ = preprocess_edges(r.src.to(dev, non_blocking=True), r.dst.to(dev, non_blocking=True), workspace=pps)
        edges += g.num_edges
        res = T.truss_decompose(g, workspace=wsp, list_budget=S.DEFAULT_LIST_BUDGET)
        plain_answers.append(S.answer_for(r.query, res.truss).cpu())
    s_plain = time.perf_counter() - t1
    reqs = [S.Request(r.id, r.arrival, r.src, r.dst, r.query) for r in base]
    srv.run(reqs, real_time=True)
    for r, a in zip(reqs, plain_answers):
        if not torch.equal(r.answer, a):
            raise SystemExit("served answer of small request %d differs from the request run alone" % r.id)
    st = S.latency_stats(reqs)
    span = max(r.t_done for r in reqs) - min(r.arrival for r in reqs)
    return {"workload": "the 4096 BA graphs of the batched section as a Poisson request stream (%.0f/s), half "
                        "decompose, half k-truss" % rate,
            "requests": num_graphs, "edges": edges, "value": edges / span, "unit": UNIT,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "makespan_s": span,
            "plain_value": edges / s_plain, "plain_s": s_plain, "speedup_vs_plain": (edges / span) / (edges / s_plain),
            "results_identical_to_plain": True}


# ---------------------------------------------------------------- GPU arm
# DRAM bytes per triangle of each phase of a decomposition (the sum of
# dram__bytes_read.sum + dram__bytes_write.sum over the phase's kernels), from
# a one-pass ncu capture of the main launches of one R-MAT scale-20
# decomposition (T = 423,980,669) of this build.  The lists, the staging area
# and the peel's slots all grow with T, so a phase's traffic at another size
# is its rate x T.  Reported beside the algorithmic bytes, never used for them.
TRAFFIC_PER_TRIANGLE = {"support": 41.2, "listing": 66.4, "peel": 46.6}
TRAFFIC_SOURCE = ("ncu one-pass capture (dram__bytes_read.sum + dram__bytes_write.sum) of one R-MAT scale-20 "
                  "decomposition, scaled per triangle")
# The same DRAM bytes per decomposition of R-MAT scale 22, edge factor 16,
# from one-kernel, one-launch, one-pass captures of the main kernels at that
# size (the one walk 130.8 GB, compaction 82.7 GB, transpose 56.0 GB, peel
# 121.3 GB; the in-adjacency and bounds kernels scaled from scale 20): at
# this size the peel's supports no longer fit in L2, so its rate per
# triangle is higher than at scale 20.
TRAFFIC_BY_WORKLOAD = {(22, 16): {"support": 133.1e9, "listing": 138.7e9, "peel": 121.3e9}}
TRAFFIC_SOURCE_BY_WORKLOAD = ("ncu one-kernel, one-launch, one-pass captures (dram__bytes_read.sum + "
                              "dram__bytes_write.sum) of the main kernels of one decomposition of this workload")


def main_ours(args):
    import torch
    ws, rank, local = dist_env()
    dist_init(ws, "nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from tdtdecomposition_gb300 import _lib, generators as G, truss as T
    from tdtdecomposition_gb300.preprocess import preprocess_edges, wedge_work
    L = _lib.load()  # raises if the CUDA library is missing

    scale, ef = args.scale, args.edge_factor
    lists_arg = {"auto": "auto", "on": True, "off": False}[args.lists]
    m = ef << scale
    src, dst = G.rmat_edges_device(scale, m, seed=1, device=dev)
    g, vertices = preprocess_edges(src, dst)
    # the GPU preprocessing of the same draws (self-loops, duplicates, degree
    # rank, orientation, sorted CSR), timed once more after that first run
    pre_stream = torch.cuda.current_stream(dev)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    p0.record(pre_stream)
    g2, _ = preprocess_edges(src, dst)
    p1.record(pre_stream)
    torch.cuda.synchronize()
    pre_ms = p0.elapsed_time(p1)
    if not (torch.equal(g2.columns, g.columns) and torch.equal(g2.row_ptr, g.row_ptr)):
        raise SystemExit("preprocessing is not deterministic")
    del src, dst, g2
    torch.cuda.synchronize()
    V, E = g.num_vertices, g.num_edges
    W = wedge_work(g)
    B_sup = 4 * W + 28 * E + 4 * (V + 1)
    wsp = T.Workspace(dev)

    def step():
        return T.truss_decompose(g, workspace=wsp, sync=False, lists=lists_arg)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # correctness anchor of this run: stats of one decomposition
    res = T.truss_decompose(g, workspace=wsp, lists=lists_arg)

    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    stream = torch.cuda.current_stream(dev)
    L.tdt_profile_start(args.steps)
    n0 = L.tdt_launch_count()
    barrier(ws)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    launches = L.tdt_launch_count() - n0
    import ctypes
    phases = (ctypes.c_float * 4)()
    nc = ctypes.c_int()
    L.tdt_profile_stop(phases, ctypes.byref(nc))
    peel_clk = T.peel_clock(wsp)  # block 0's split of the last timed peel
    clk = clocks.stop() if clocks else None
    t_ms = ev0.elapsed_time(ev1)
    t_ms = max_over_ranks(t_ms, ws, dev)
    ms_step = t_ms / args.steps
    value = ws * E / (ms_step / 1e3)

    # e2e: host buffers through the public API.  The graph goes over as CSR
    # (columns + row_ptr): truss_decompose derives the COO rows on the device
    # when a CSRCOO comes without them, so they are not copied.
    cols_h = g.columns.cpu().pin_memory()
    rp_h = g.row_ptr.cpu().pin_memory()
    truss_h = torch.empty(E, dtype=torch.int32).pin_memory()
    from tdtdecomposition_gb300 import CSRCOO
    d_cols = torch.empty_like(g.columns)
    d_rp = torch.empty_like(g.row_ptr)

    e2e_stats = []

    def e2e_step():
        d_cols.copy_(cols_h, non_blocking=True)
        d_rp.copy_(rp_h, non_blocking=True)
        tr, _, _, st = T.truss_decompose(CSRCOO(columns=d_cols, row_ptr=d_rp), workspace=wsp, sync=False,
                                         lists=lists_arg)
        truss_h.copy_(tr, non_blocking=True)
        e2e_stats.append(st)

    e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    te = max_over_ranks(e0.elapsed_time(e1), ws, dev)
    bad = [st.cpu().tolist() for st in e2e_stats if int(st[0]) != 0]
    ref_truss = res.truss.cpu()
    if bad or not torch.equal(truss_h, ref_truss):
        ndiff = int((truss_h != ref_truss).sum())
        print(json.dumps({"error": "e2e result differs from the resident run", "differing_edges": ndiff,
                          "bad_stats": bad[:3], "resident_stats": [res.kmax, res.triangles, res.rounds]}),
              file=sys.stderr, flush=True)
        raise SystemExit(3)
    e2e_value = ws * E / (te / args.steps / 1e3)
    h2d = cols_h.numel() * 4 + rp_h.numel() * 8
    d2h = truss_h.numel() * 4

    if rank != 0:
        return
    peak, peak_src = _hbm_peak()
    n = max(nc.value, 1)
    t_sup, t_list, t_peel, t_post = (phases[k] / n for k in range(4))
    # the decomposition's algorithmic bytes B_dec = 2 B_sup: the support pass,
    # then one re-enumeration of each edge's triangles (listing + peel)
    mt = TRAFFIC_BY_WORKLOAD.get((scale, ef)) or {k: v * res.triangles for k, v in TRAFFIC_PER_TRIANGLE.items()}
    traffic_src = TRAFFIC_SOURCE_BY_WORKLOAD if (scale, ef) in TRAFFIC_BY_WORKLOAD else TRAFFIC_SOURCE
    if res.listing != 2:
        # the captures behind these figures are of the one-walk listed path
        mt, traffic_src = None, "not captured for this path"
    B_dec = 2 * B_sup
    ach = B_dec / (ms_step / 1e3) / 1e9
    phases_ms = {"support": t_sup, "listing": t_list, "peel": t_peel, "outputs": t_post}
    per_kernel = {
        "support_kernel": {"ms": round(t_sup, 4), "algorithmic_bytes": B_sup,
                           "achieved_gbs": round(B_sup / (t_sup / 1e3) / 1e9, 1),
                           "traffic": mt["support"] if mt else None},
        "reenumeration (listing + transpose + peel kernels)": {
            "ms": round(t_list + t_peel, 4), "algorithmic_bytes": B_sup,
            "achieved_gbs": round(B_sup / ((t_list + t_peel) / 1e3) / 1e9, 1),
            "traffic": (mt["listing"] + mt["peel"]) if mt else None},
        "peel_kernel": {"ms": round(t_peel, 4), "traffic": mt["peel"] if mt else None,
                        "dram_gbs": round(mt["peel"] / (t_peel / 1e3) / 1e9, 1) if mt else None},
    }
    roof = {"bound": "hbm", "kernel": "decomposition (all kernels of one step)", "achieved": ach, "peak": peak,
            "unit": "GB/s", "frac": ach / peak, "traffic": sum(mt.values()) if mt else None,
            "algorithmic_bytes": B_dec, "peak_source": peak_src, "per_kernel": per_kernel, "phase_ms": phases_ms,
            "peel_clock_ms": {k: round(v, 2) for k, v in peel_clk.items()},
            "traffic_source": traffic_src}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "R-MAT scale %d edge factor %d single-graph truss decomposition" % (scale, ef),
                       "scale": scale, "edge_factor": ef, "abcd": [0.57, 0.19, 0.19, 0.05], "seed": 1,
                       "V": V, "E": E, "W": W, "kmax": res.kmax, "triangles": res.triangles,
                       "rounds": res.rounds, "parallelism": "replicas" if ws > 1 else "single",
                       "triangle_lists": {2: "one walk counts and lists (listed peel)",
                                          1: "count walk + listing walk (listed peel)"}.get(
                                              res.listing, "none (search peel)"),
                       "l2": "inputs larger than L2 (CSR %.0f MB + in-adjacency)" % ((8 * E + 8 * V) / 1e6)},
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": te / args.steps},
            "preprocess": {"draws": m, "ms": pre_ms, "draws_per_s": m / (pre_ms / 1e3),
                           "what": "R-MAT draws (device-resident) -> deduplicated degree-oriented CSR, "
                                   "tdt_preprocess (radix sorts, scans, relabel)"},
            "gpu_launches": int(launches), "clocks": clk}
    if not args.no_batched:
        line["batched"] = bench_batched(dev, args.steps, args.warmup)
    if not args.no_served:
        line["served"] = bench_served(dev)
    # the benchmark's workspace (lists and staging, most of the device) goes
    # before the other sections allocate theirs
    wsp.buf = None
    torch.cuda.empty_cache()
    if not args.no_reference_gpu:
        line["reference_gpu"] = bench_reference_gpu(dev, g, wsp)
        wsp.buf = None
        torch.cuda.empty_cache()
    if not args.no_skewed:
        line["skewed"] = bench_skewed(dev, args.skewed_log2n)
        torch.cuda.empty_cache()
    if args.fusion:
        line["fusion"] = bench_fusion(dev, args.fusion_scale)
    if args.undirected:
        line["undirected"] = bench_undirected(dev, args.fusion_scale)
    sc = cpu_sample_scale(args, args.steps + args.warmup)
    same, gpu_truss = (None, None) if args.no_same_scale else bench_same_scale(dev, sc, args.steps)
    if not args.no_cpu_baseline:
        import numpy as np
        Ec, Vc, times, threads, cpu_truss = cpu_decompose_sample(sc, 1)
        line["cpu_baseline"] = {"value": Ec / times[0], "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "R-MAT scale %d, 16*2^%d draws, seed 1 (V=%d, E=%d), one full "
                                          "decomposition, %.1f s" % (sc, sc, Vc, Ec, times[0])}
        if same is not None:
            same["cpu_value"] = Ec / times[0]
            same["cpu_kind"] = "port (oracle restatement of the --cuda flow, OpenMP, %d threads)" % threads
            same["gpu_over_cpu"] = same["gpu_value"] / same["cpu_value"]
            same["results_identical"] = bool(np.array_equal(gpu_truss, cpu_truss))
    if same is not None:
        line["same_scale"] = same
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        main_ours(args)


if __name__ == "__main__":
    main()
