"""Benchmark of the hypervector classification hot path on GB300.

A step is one batch of synthetic reads pushed through the hot path with the
reference database resident in HBM: encode every read (kernel a), then
exact cosine top-k against every reference (kernel b).  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c1|c2|c3|c4|c5|aux]
                    [--form plain|tc] [--batch B] [--impl ours|reference]

Workloads (seeded synthetic data standing in for real 16S data, none of
which is available here):
  c1  the reference's CPU-runnable case: 2,000 leaf references, D=8192, k=8, the
      10,000 reads of 150 bp (1% substitutions) as one step, top-5; the result is
      compared with the compiled reference's own answers for the same workload
  c2  plain GPU drop-in at scale: 50,000 leaf references of a 6-rank tree,
      D=8192, k=8, reads of 150 bp with 1% substitutions, top-5, NORM score
  c3  precision form: 200,000 leaf references, each the bundle of 8 noisy
      copies (1% substitutions) of its leaf, D=10240, k=10; reads of 250 bp
      with 1% substitutions, bipolar queries, top-5
  c4  batching form: c3's database, reads of log-normal length (100-1600 bp),
      20% with 6% substitutions and indels, top-10, CUDA-graph pipeline
  c5  hierarchical descent: 500,000 leaves + every internal prototype of a
      6-rank tree, D=16384, k=12, c4's reads, top-5 per rank root to leaf;
      a step is the read encode and the descent (two cooperative launches by
      default; --beam-one selects the other forms)
  aux the kernels beside the hot path (FASTA ingest, packing, similarity,
      identify, greedy selection), each timed once

--impl reference times the reference CPU algorithm (the C restatement in
oracle/, the reference's own sources being unavailable on the GPU host) on
the host cores, on a bounded sample of the same workload.

The library is single-GPU: its tensor-core search multicasts operand tiles
between the CTAs of a cluster, within the calling GPU's own memory only.
Launched with WORLD_SIZE > 1 the benchmark does no work: rank 0 prints an
"unavailable" line and every rank exits 0.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bacterial-classification_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

CONFIGS = {
    # the reference's CPU-runnable case: 2,000 leaves, 10,000 reads of 150 bp a step (the whole workload),
    # checked against the compiled reference's own top-5 (tests/golden/c1_known_answer.json)
    "c1": dict(n_leaves=2000, dim=8192, kmer=8, read_len=150, subst=0.01, topk=5, copies=0, bipolar=False,
               tree_seed=1, read_seed=101, copy_seed=0, batch=10000, known_answer="c1_known_answer.json"),
    "c2": dict(n_leaves=50000, dim=8192, kmer=8, read_len=150, subst=0.01, topk=5, copies=0, bipolar=False,
               tree_seed=2, read_seed=102, copy_seed=0),
    "c3": dict(n_leaves=200000, dim=10240, kmer=10, read_len=250, subst=0.01, topk=5, copies=8, bipolar=True,
               tree_seed=3, read_seed=103, copy_seed=203),
    # batching form: the config-3 database, reads of log-normal length (median 250, sigma 0.5,
    # clipped to 100-1600), 20 % of them with 6 % substitution:insertion:deletion = 3:1:1 errors
    "c4": dict(n_leaves=200000, dim=10240, kmer=10, read_len=250, subst=0.01, topk=10, copies=8, bipolar=True,
               tree_seed=3, read_seed=104, copy_seed=203, sigma=0.5, min_read=100, max_read=1600,
               mixed_frac=0.2, mixed_rate=0.06),
    # hierarchical descent: 500,000 leaves + internal prototypes (exact int32 sums of their
    # children, bottom-up over the 6 ranks), D=16,384, k=12; config-4 read distribution;
    # beam 5 per rank, root to leaf (no early stop), in two cooperative launches per batch
    "c5": dict(n_leaves=500000, dim=16384, kmer=12, read_len=250, subst=0.01, topk=5, copies=0, bipolar=True,
               tree_seed=5, read_seed=105, sigma=0.5, min_read=100, max_read=1600, mixed_frac=0.2,
               mixed_rate=0.06, beam=5, levels=6, threshold=float("-inf")),
}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the
# dominant kernel, from single-pass ncu captures of the full-size workloads, per
# unit of work, so a run's `traffic` is that per-unit figure times its own units:
#   tc_search_kernel, c3 (38,912 reads x 200,000 refs = 304 x 1,564 tile pairs; the
#     288 leading query tiles in clusters of 4 + the other 16 in pairs): 1.01427e12 B
#   grouped descent, c5 (one call's 5 descent_tc_kernel launches + the leaf-level score_kernel,
#     38,912 reads): 3.64798e10 B with every row int32, 2.03567e10 B with int16 leaf rows
TRAFFIC_PER_TILE_PAIR_TC = (975.445256e9 + 0.170780e9 + 38.640838e9 + 0.012020e9) / (304 * 1564)
# (reads per call, int16 rows) -> bytes (mostly the database, once)
TRAFFIC_DESCENT = {(38912, False): 36.409726e9 + 70.093e6, (38912, True): 2.035667e10}


# the CPU port against the reference's own compiled code, both on one x86 thread at the c3 shape
# (D = 10,240, k = 10, 250 bp reads, 2,000 references): 48.8 vs 64.8 reads/s
PORT_NOTE = ("the oracle port of the reference's CPU path (its sources are not on this host); on x86 the "
             "port ran at 0.75x the compiled reference (48.8 vs 64.8 reads/s, one thread, c3 shape)")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, \
        "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---------------------------------------------------------------------------- workload
def build_database(H, ctx, cfg, dev):
    """Reference hypervectors resident in HBM: leaves (c2) or bundles of noisy copies (c3)."""
    import torch
    t0 = time.time()
    tree = H.synth_tree(cfg["tree_seed"], cfg["n_leaves"])
    nr, dim = cfg["n_leaves"], cfg["dim"]
    refs = torch.empty((nr, dim), dtype=torch.int16, device=dev)
    d_tree = torch.from_numpy(tree.buf).to(dev)
    chunk = 8192
    for a in range(0, nr, chunk):
        b = min(nr, a + chunk)
        sub = H.Seqs(tree.buf, tree.off[a:b], tree.len[a:b])
        if cfg["copies"]:
            cp = H.synth_copies(cfg["copy_seed"] + a, sub, cfg["copies"], 0.01)
            d_b = torch.from_numpy(cp.buf).to(dev)
            n = len(cp)
            tmp = torch.empty((n, dim), dtype=torch.int32, device=dev)
            ctx.encode_segments(d_b, torch.from_numpy(cp.off).to(dev), torch.from_numpy(cp.len).to(dev), tmp,
                                H.OUT_I32, cp.max_len())
            ptr = torch.arange(0, n + 1, cfg["copies"], dtype=torch.int64, device=dev)
            idx = torch.arange(n, dtype=torch.int32, device=dev)
            summed = ctx.bundle(tmp, ptr, idx)
            refs[a:b] = summed.to(torch.int16)  # |sum| <= 8 * 1600 fits int16
        else:
            off = torch.from_numpy(np.ascontiguousarray(tree.off[a:b])).to(dev)
            ln = torch.from_numpy(np.ascontiguousarray(tree.len[a:b])).to(dev)
            ctx.encode_segments(d_tree, off, ln, refs[a:b], H.OUT_I16, int(tree.len[a:b].max()))
    maxr = torch.zeros(1, dtype=torch.int32, device=dev)
    rn = ctx.norms(refs, maxr)
    torch.cuda.synchronize()
    log("database: %d references x %d dims built in %.1f s" % (nr, dim, time.time() - t0))
    return tree, refs, rn, int(maxr.item())


def known_answer(cfg, idx, score):
    """The batch's top-k indices and float scores against the compiled reference's answers for the same
    workload (sha256 of int32 / float32 little-endian arrays, as tests/golden/make_c1_golden.py stores them)."""
    import hashlib
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", cfg["known_answer"])))
    h = lambda a: hashlib.sha256(a.tobytes()).hexdigest()
    n = gold["workload"]["n_reads"]
    if idx.shape[0] != n:
        return {"identical": None, "note": "the known answers cover exactly %d reads" % n}
    i_ok = h(np.ascontiguousarray(idx, "<i4")) == gold["idx_sha256"]
    s_ok = h(np.ascontiguousarray(score, "<f4")) == gold["score_sha256"]
    return {"indices_identical": bool(i_ok), "float_scores_identical": bool(s_ok), "identical": bool(i_ok and s_ok),
            "source": gold["source"]}


def make_reads(H, tree, cfg, n, seed):
    return H.synth_reads(seed, tree, n, cfg["read_len"], subst=cfg["subst"], sigma=cfg.get("sigma", 0.0),
                         min_read=cfg.get("min_read", 100), max_read=cfg.get("max_read", 1600),
                         mixed_frac=cfg.get("mixed_frac", 0.0), mixed_rate=cfg.get("mixed_rate", 0.0))


# ---------------------------------------------------------------------------- our arm
class Form:
    """One GPU form of the hot path for a fixed batch size: encode the batch of
    reads, then top-k search against the resident database.
      plain: int16 queries (counts, or +1/-1 when the workload is bipolar),
             exact search on CUDA cores (hdc_search_plain)
      tc:    fp16 queries (+1/-1, or counts when the workload is not bipolar), exact
             search on tcgen05 tensor cores (hdc_search_tc against an fp16-limb
             database whose limbs are sized for the largest query magnitude)"""

    def __init__(self, H, ctx, cfg, name, refs, rn, maxr, B, dev, db=None):
        import torch
        self.H, self.ctx, self.cfg, self.name, self.B = H, ctx, cfg, name, B
        self.refs, self.rn, self.maxr = refs, rn, maxr
        K, dim = cfg["topk"], cfg["dim"]
        self.K = K
        if name == "tc":
            if cfg["bipolar"]:
                self.db = db if db is not None else ctx.refdb(refs, maxr)
                self.kind, self.maxq = H.OUT_BIPOLAR_F16, 1
            else:  # count-valued reads: fp16 counts, limbs sized for them
                self.maxq = cfg["read_len"] - cfg["kmer"] + 1
                self.db = ctx.refdb(refs, maxr, max_query_abs=self.maxq)
                self.kind = H.OUT_F16
            self.q = torch.empty((B, dim), dtype=torch.float16, device=dev)
            self.work = torch.empty(max(16, H.lib().hdc_search_tc_workspace_bytes(ctx.h, self.db.h, B, K)),
                                    dtype=torch.uint8, device=dev)
        else:
            self.db = None
            self.kind = H.OUT_BIPOLAR_I16 if cfg["bipolar"] else H.OUT_I16
            self.q = torch.empty((B, dim), dtype=torch.int16, device=dev)
            self.maxq = 1 if cfg["bipolar"] else cfg["read_len"] - cfg["kmer"] + 1
            self.work = torch.empty(max(16, ctx.workspace_bytes(B, refs.shape[0], K)), dtype=torch.uint8,
                                    device=dev)
        # +1/-1 rows have squared norm dim exactly; count rows are normed per batch
        self.qn = torch.full((B,), dim, dtype=torch.int64, device=dev) if cfg["bipolar"] else None
        self.out = (torch.empty((B, K), dtype=torch.float32, device=dev),
                    torch.empty((B, K), dtype=torch.int32, device=dev),
                    torch.empty((B, K), dtype=torch.float64, device=dev),
                    torch.empty((B, K), dtype=torch.int64, device=dev))
        self.launches = 3 if cfg["bipolar"] else 4  # encode, [norms], search, merge
        # the reference's NORM scale by default; --score-mode dot/cos for kernel studies
        self.mode = {"norm": H.SCORE_NORM, "cos": H.SCORE_COS, "dot": H.SCORE_DOT}[cfg.get("score_mode", "norm")]

    def run(self, buf, off, ln, ev=None, stream=None):
        H, ctx = self.H, self.ctx
        ctx.encode_segments(buf, off, ln, self.q, self.kind, self.cfg["read_len"])
        qn = self.qn if self.qn is not None else ctx.norms(self.q)
        if ev is not None:
            ev[0].record(stream)
        if self.name == "tc":
            ctx.search_tc(self.db, self.q, qn, 1, self.K, self.mode, work=self.work, out=self.out)
            # encode, [norms], then the search kernels and merges the library reports (one or two parts)
            self.launches = (1 if self.cfg["bipolar"] else 2) + ctx.tc_last_shape()[4]
        else:
            ctx.search_plain(self.q, qn, self.maxq, self.refs, self.rn, self.maxr, self.K, self.mode,
                             work=self.work, out=self.out)
        if ev is not None:
            ev[1].record(stream)
        return self.out


def time_form(form, batches, d_buf, steps, warmup, sampler=None):
    """Device-timed steps of one form on resident batches; also the median
    duration of its search kernel (+ merge) alone, on the same stream."""
    import torch
    stream = torch.cuda.current_stream()
    for i in range(warmup):
        form.run(d_buf, *batches[i % len(batches)])
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctxm = sampler if sampler is not None else _Null()
    with ctxm:
        torch.cuda.synchronize()
        t0.record(stream)
        for i in range(steps):
            form.run(d_buf, *batches[i % len(batches)])
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    ev = [torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
    search = []
    for i in range(3):
        form.run(d_buf, *batches[i % len(batches)], ev=ev, stream=stream)
        torch.cuda.synchronize()
        search.append(ev[0].elapsed_time(ev[1]))
    return ms, float(np.median(search))


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def run_pipeline(args, cfg, H, ctx, tree, refs, rn, maxr, dev, db=None):
    """Batching form: the CUDA-graph pipeline over host batches of uneven reads
    (against `db` when the tensor-core database is already built)."""
    import torch
    B, K = args.batch, cfg["topk"]
    pool = [make_reads(H, tree, cfg, B, cfg["read_seed"] + p) for p in range(2)]
    max_bytes = max(int(r.len.astype(np.int64).sum()) for r in pool) + 4096
    if db is None:
        db = ctx.refdb(refs, maxr)
    pipe = H.Pipeline(ctx, db, B, max_bytes, cfg.get("max_read", cfg["read_len"]), K)
    pipe.run(pool[0])
    tuned = pipe.autotune()
    # device-resident: replay encode + search on the staged batch, timed on the pipeline's stream
    st = torch.cuda.ExternalStream(pipe.stream())
    for _ in range(args.warmup):
        pipe.launch_resident()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(dev.index)
    with clk:
        e0.record(st)
        for _ in range(args.steps):
            pipe.launch_resident()
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # end to end: host batches through hdc_pipeline_run (host packing, copies, graph, copies back)
    for i in range(args.warmup):
        pipe.run(pool[i % 2])
    t0 = time.perf_counter()
    for i in range(args.steps):
        pipe.run(pool[i % 2])
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    # the timed schedule's results on the first batch: accuracy, and the oracle's parity sample
    first_s, first_idx = pipe.run(pool[0])
    acc = float((first_idx[:, 0] == pool[0].label).mean())
    # each graph replay runs encode_kernel, then the search and merge kernels of each part of the
    # search (memset nodes aside): the search the graph captured after the autotune
    per_step = 1 + ctx.tc_last_shape()[4]
    # the search kernel alone on the same batch, for the roofline
    form = Form(H, ctx, cfg, "tc", refs, rn, maxr, B, dev, db=db)
    d_buf = torch.from_numpy(pool[0].buf).to(dev)
    bat = [(torch.from_numpy(pool[0].off).to(dev), torch.from_numpy(pool[0].len).to(dev))]
    _, search_ms = time_form(form, bat, d_buf, 2, 3)
    return dict(ms=ms, e2e_ms=e2e_ms, search_ms=search_ms, clocks=clk.summary(), launches=per_step * args.steps,
                refs=refs.shape[0], limbs=db.limbs, h2d=max_bytes + B * 16, d2h=B * K * 8, tree=tree,
                tuned=tuned, mean_len=float(np.mean(pool[0].len)), top1_accuracy=acc,
                refs_host=refs.cpu().numpy() if not args.no_cpu_baseline else None, reads=pool[0],
                gpu_first=(first_s[:1024], first_idx[:1024], None, None))


def run_ours(args, cfg):
    import torch
    import hdc_gb300 as H
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = H.Context(cfg["dim"], cfg["kmer"], cfg["read_len"], 10)
    if args.tc_group or args.tc_cluster:
        ctx.tc_tuning(args.tc_group, -1, 0, 0)
        ctx.tc_option(H.TC_CLUSTER, args.tc_cluster)
    tree, refs, rn, maxr = build_database(H, ctx, cfg, dev)
    if args.form == "pipe":
        return run_pipeline(args, cfg, H, ctx, tree, refs, rn, maxr, dev)
    B = args.batch
    n_pool = 2
    reads = make_reads(H, tree, cfg, B * n_pool, cfg["read_seed"])
    d_buf = torch.from_numpy(reads.buf).to(dev)
    batches = []
    for p in range(n_pool):
        off = torch.from_numpy(np.ascontiguousarray(reads.off[p * B:(p + 1) * B])).to(dev)
        ln = torch.from_numpy(np.ascontiguousarray(reads.len[p * B:(p + 1) * B])).to(dev)
        batches.append((off, ln))
    form = Form(H, ctx, cfg, args.form, refs, rn, maxr, B, dev)
    clk = ClockSampler(dev.index)
    ms, search_ms = time_form(form, batches, d_buf, args.steps, args.warmup, clk)
    res = dict(ms=ms, search_ms=search_ms, clocks=clk.summary(), launches=form.launches * args.steps,
               refs=refs.shape[0], limbs=form.db.limbs if form.db is not None else 0)
    # the source leaf of every read is known: how often is it the top hit
    form.run(d_buf, *batches[0])
    torch.cuda.synchronize()
    res["top1_accuracy"] = float((form.out[1][:B, 0].cpu().numpy() == reads.label[:B]).mean())
    res["gpu_first"] = tuple(x[:1024].cpu().numpy() for x in form.out)  # for the oracle's parity sample
    res["reads"] = reads
    if cfg.get("known_answer"):
        res["known_answer"] = {"form": form.name, "reads": B}
        res["known_answer"].update(known_answer(cfg, form.out[1][:B].cpu().numpy(), form.out[0][:B].cpu().numpy()))

    # the plain drop-in on the same workload, for the tensor-core speed-up
    if args.form == "tc" and not args.no_plain:
        pb = min(B, args.plain_batch)
        pbat = [(o[:pb], l[:pb]) for o, l in batches]
        plain = Form(H, ctx, cfg, "plain", refs, rn, maxr, pb, dev)
        pms, psearch = time_form(plain, pbat, d_buf, max(2, args.steps // 2), 3)
        res["plain"] = dict(value=pb / (pms / 1e3), ms=pms, batch=pb, search_ms=psearch)
        del plain
        # identical labels: the first plain batch against the tensor-core result
        form.run(d_buf, *pbat[0])
        tc_idx = form.out[1][:pb].clone()
        plain2 = Form(H, ctx, cfg, "plain", refs, rn, maxr, pb, dev)
        plain2.run(d_buf, *pbat[0])
        torch.cuda.synchronize()
        res["labels_identical_to_plain"] = bool(torch.equal(tc_idx, plain2.out[1]))
        del plain2

    # the precision form on the plain drop-in's workload (count-valued reads), for the speed-up
    if args.form == "plain" and not cfg["bipolar"] and not args.no_plain:
        tcf = Form(H, ctx, cfg, "tc", refs, rn, maxr, B, dev)
        tms, tsearch = time_form(tcf, batches, d_buf, max(2, args.steps // 2), 3)
        tcf.run(d_buf, *batches[0])
        form.run(d_buf, *batches[0])
        torch.cuda.synchronize()
        if cfg.get("known_answer"):
            res["tc_known_answer"] = known_answer(cfg, tcf.out[1][:B].cpu().numpy(), tcf.out[0][:B].cpu().numpy())
        res["tc_form"] = dict(value=B / (tms / 1e3), ms=tms, search_ms=tsearch, limbs=tcf.db.limbs,
                              limb_bits=tcf.db.limb_bits,
                              labels_identical=bool(torch.equal(tcf.out[1], form.out[1])),
                              scores_identical=bool(torch.equal(tcf.out[0], form.out[0])))
        del tcf

    # end to end through the C ABI with pinned host buffers, copies inside the timed region
    stream = torch.cuda.current_stream()
    h_bufs = []
    for p in range(n_pool):
        o0 = int(reads.off[p * B])
        o1 = int(reads.off[(p + 1) * B - 1] + reads.len[(p + 1) * B - 1])
        hb = torch.from_numpy(reads.buf[o0:o1].copy()).pin_memory()
        ho = torch.from_numpy(reads.off[p * B:(p + 1) * B] - o0).pin_memory()
        hl = torch.from_numpy(reads.len[p * B:(p + 1) * B].copy()).pin_memory()
        h_bufs.append((hb, ho, hl))
    cap = max(x[0].numel() for x in h_bufs)
    e_buf = torch.empty(cap + 16, dtype=torch.uint8, device=dev)
    e_off = torch.empty(B, dtype=torch.int64, device=dev)
    e_len = torch.empty(B, dtype=torch.int32, device=dev)
    h_s = torch.empty((B, form.K), dtype=torch.float32).pin_memory()
    h_i = torch.empty((B, form.K), dtype=torch.int32).pin_memory()
    io = {}

    def e2e_step(i):
        hb, ho, hl = h_bufs[i % n_pool]
        e_buf[:hb.numel()].copy_(hb, non_blocking=True)
        e_off.copy_(ho, non_blocking=True)
        e_len.copy_(hl, non_blocking=True)
        out = form.run(e_buf, e_off, e_len)
        h_s.copy_(out[0], non_blocking=True)
        h_i.copy_(out[1], non_blocking=True)
        io["h2d"] = hb.numel() + ho.numel() * 8 + hl.numel() * 4
        io["d2h"] = h_s.numel() * 4 + h_i.numel() * 4

    for i in range(args.warmup):
        e2e_step(i)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(args.steps):
        e2e_step(i)
    t1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / args.steps
    res.update(e2e_ms=e2e_ms, h2d=io["h2d"], d2h=io["d2h"], tree=tree)
    res["refs_host"] = refs.cpu().numpy() if not args.no_cpu_baseline else None

    # the batching form on the same database: the c4 reads (log-normal lengths, 20 % with mixed
    # errors, top-10) through the CUDA-graph pipeline, after its autotune
    if args.form == "tc" and cfg["copies"] and not args.no_batching:
        c4 = dict(CONFIGS["c4"], n_leaves=cfg["n_leaves"])
        res["batching"] = run_pipeline(args, c4, H, ctx, tree, refs, rn, maxr, dev, db=form.db)
        res["batching"]["cfg"] = c4
    return res


def build_prototypes(H, ctx, cfg, dev):
    """Taxonomy prototypes resident in HBM: leaf encodings (int32) and every
    internal node the exact int32 sum of its children (hdc_bundle, rank by
    rank from the leaves up).  Also the bundle kernel's timing per rank."""
    import torch
    t0 = time.time()
    tree = H.synth_tree(cfg["tree_seed"], cfg["n_leaves"])
    b, base, counts, ptr, idx = H.synth_tree_csr(cfg["n_leaves"])
    n_nodes, dim = int(base[-1]), cfg["dim"]
    proto = torch.empty((n_nodes, dim), dtype=torch.int32, device=dev)
    d_tree = torch.from_numpy(tree.buf).to(dev)
    leaf0 = int(base[5])
    chunk = 16384
    for a in range(0, cfg["n_leaves"], chunk):
        e = min(cfg["n_leaves"], a + chunk)
        off = torch.from_numpy(np.ascontiguousarray(tree.off[a:e])).to(dev)
        ln = torch.from_numpy(np.ascontiguousarray(tree.len[a:e])).to(dev)
        ctx.encode_segments(d_tree, off, ln, proto[leaf0 + a:leaf0 + e], H.OUT_I32, int(tree.len[a:e].max()))
    d_idx = torch.from_numpy(idx).to(dev)
    bundle = []
    for r in range(4, -1, -1):
        lo, hi = int(base[r]), int(base[r + 1])
        cp = torch.from_numpy(ptr[lo:hi + 1].copy()).to(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.bundle(proto, cp, d_idx, out=proto[lo:hi])
        e1.record()
        torch.cuda.synchronize()
        n_child = int(ptr[hi] - ptr[lo])
        bundle.append(dict(rank=r + 1, parents=hi - lo, children=n_child, ms=e0.elapsed_time(e1),
                           bytes=(n_child + hi - lo) * dim * 4))
    pn = ctx.norms(proto)
    torch.cuda.synchronize()
    log("prototypes: %d nodes x %d dims (%.1f GB) built in %.1f s" % (n_nodes, dim, n_nodes * dim * 4 / 1e9,
                                                                   time.time() - t0))
    return tree, proto, pn, (b, base, counts, ptr, idx), bundle


def run_descent(args, cfg):
    """Hierarchical descent: per step, encode a batch of reads to +1/-1 int8
    and run the beam descent over the resident prototypes."""
    import torch
    import hdc_gb300 as H
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    dim, B, L, W = cfg["dim"], args.batch, cfg["levels"], cfg["beam"]
    ctx = H.Context(dim, cfg["kmer"], cfg["read_len"], 10)
    ctx.option(H.BEAM_GROUPED, args.beam_grouped)
    ctx.option(H.BEAM_ONE_LAUNCH, args.beam_one)
    tree, proto, pn, (b, base, counts, ptr, idx), bundle = build_prototypes(H, ctx, cfg, dev)
    d_ptr, d_idx = torch.from_numpy(ptr).to(dev), torch.from_numpy(idx).to(dev)
    roots = torch.arange(0, counts[0], dtype=torch.int32, device=dev)
    n_nodes = proto.shape[0]
    max_children = int(np.diff(ptr).max())
    # the leaves are scored from an int16 copy of their rows (hdc_beam_search_split) when they
    # fit 16 bits (whole-sequence counts): their level streams its rows from HBM, so it reads
    # half the bytes.  The ranks above stay int32: the tensor-core levels are bound by their
    # producers' conversions, not by bytes, and an int32 row converts in fewer instructions.
    split = not args.proto_int32 and args.beam_grouped != 0 and dim % 1024 == 0 and dim <= 16384
    n_wide = max(first_int16_row(proto), int(base[5])) if split else n_nodes
    proto32 = proto[:n_wide]
    proto16 = torch.empty((n_nodes - n_wide, dim), dtype=torch.int16, device=dev)
    for i in range(0, n_nodes - n_wide, 8192):
        proto16[i:i + 8192].copy_(proto[n_wide + i:n_wide + i + 8192])
    n_pool = 2
    pool = [make_reads(H, tree, cfg, B, cfg["read_seed"] + p) for p in range(n_pool)]
    max_len = max(r.max_len() for r in pool)
    q8 = torch.empty((B, dim), dtype=torch.int8, device=dev)
    qn = torch.full((B,), dim, dtype=torch.int64, device=dev)  # every element of a +1/-1 read is nonzero
    dev_pool = [(torch.from_numpy(r.buf).to(dev), torch.from_numpy(r.off).to(dev), torch.from_numpy(r.len).to(dev))
                for r in pool]
    out = {}

    # split form: the reads go straight to sign bits (HDC_OUT_SIGN_BITS, hdc_beam_search_split_bits)
    qbits = torch.empty((B, dim // 32), dtype=torch.int32, device=dev) if split else None

    def step(d_buf, d_off, d_len, ev=None):
        if split:
            ctx.encode_segments(d_buf, d_off, d_len, qbits, H.OUT_SIGN_BITS, max_len)
        else:
            ctx.encode_segments(d_buf, d_off, d_len, q8, H.OUT_BIPOLAR_I8, max_len)
        if ev:
            ev[0].record()
        if split:  # the tree's largest child count is known here: no host synchronisation in the call
            out["r"] = ctx.beam_search_split(qbits, qn, proto32, proto16, pn, d_ptr, d_idx, roots, L, W,
                                             cfg["threshold"], max_children=max_children)
        else:
            out["r"] = ctx.beam_search(q8, qn, proto, pn, d_ptr, d_idx, roots, L, W, cfg["threshold"])
        if ev:
            ev[1].record()
        return out["r"]

    for i in range(args.warmup):
        step(*dev_pool[i % n_pool])
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(dev.index)
    with clk:
        torch.cuda.synchronize()
        t0.record(stream)
        for i in range(args.steps):
            step(*dev_pool[i % n_pool])
        t1.record(stream)
        torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    ev = [torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
    beam_ms = []
    for i in range(3):
        step(*dev_pool[i % n_pool], ev=ev)
        torch.cuda.synchronize()
        beam_ms.append(ev[0].elapsed_time(ev[1]))
    path, score, depth = out["r"]
    phases = descent_phases(ctx.beam_phase_times(), L, grouped_tc=args.beam_grouped in (-1, 2),
                            apart=args.beam_one != 1) if split and args.beam_one != 0 else None
    depth_mean = float(depth.float().mean())
    last = 2 % n_pool  # out["r"] is from the last event-timed call, on dev_pool[2 % n_pool]
    leaf_acc = float((path[:, L - 1].cpu().numpy() == int(base[5]) + pool[last].label[:B]).mean())
    # the same calls as kernels per level (HDC_BEAM_ONE_LAUNCH 0), timed beside the form above
    alt = None
    if split and args.beam_one != 0:
        ref = [x.clone() for x in (path, score, depth)]
        ctx.option(H.BEAM_ONE_LAUNCH, 0)
        for i in range(args.warmup):
            step(*dev_pool[i % n_pool])
        torch.cuda.synchronize()
        t0.record(stream)
        for i in range(args.steps):
            step(*dev_pool[i % n_pool])
        t1.record(stream)
        torch.cuda.synchronize()
        alt_ms = t0.elapsed_time(t1) / args.steps
        step(*dev_pool[last])
        torch.cuda.synchronize()
        same = all(torch.equal(x, y) for x, y in zip(ref, out["r"]))
        alt = {"form": "kernels per level (HDC_BEAM_ONE_LAUNCH 0)", "value": B / (alt_ms / 1e3), "unit": "reads/s",
               "ms_per_step": alt_ms, "gpu_launches_per_step": 1 + 3 + 6 * L + 2 + 14 * (L - 2) + 5,
               "results_identical": same}
        ctx.option(H.BEAM_ONE_LAUNCH, args.beam_one)
    # end to end: pinned host reads copied in, paths and scores copied back, every step
    h_pool = [(torch.from_numpy(r.buf).pin_memory(), torch.from_numpy(r.off).pin_memory(),
               torch.from_numpy(r.len).pin_memory()) for r in pool]
    cap = max(h[0].numel() for h in h_pool)
    e_buf = torch.empty(cap, dtype=torch.uint8, device=dev)
    e_off = torch.empty(B, dtype=torch.int64, device=dev)
    e_len = torch.empty(B, dtype=torch.int32, device=dev)
    h_path = torch.empty((B, L), dtype=torch.int32).pin_memory()
    h_score = torch.empty((B, L), dtype=torch.float32).pin_memory()
    io = {}

    def e2e_step(i):
        hb, ho, hl = h_pool[i % n_pool]
        e_buf[:hb.numel()].copy_(hb, non_blocking=True)
        e_off.copy_(ho, non_blocking=True)
        e_len.copy_(hl, non_blocking=True)
        p, s_, _ = step(e_buf, e_off, e_len)
        h_path.copy_(p, non_blocking=True)
        h_score.copy_(s_, non_blocking=True)
        io["h2d"] = hb.numel() + ho.numel() * 8 + hl.numel() * 4
        io["d2h"] = h_path.numel() * 4 + h_score.numel() * 4

    for i in range(args.warmup):
        e2e_step(i)
    torch.cuda.synchronize()
    t0.record(stream)
    for i in range(args.steps):
        e2e_step(i)
    t1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / args.steps
    if split:  # the last step's reads as int8 rows too (untimed), for the oracle's sample
        ctx.encode_segments(e_buf, e_off, e_len, q8, H.OUT_BIPOLAR_I8, max_len)
    # candidate rows per read: the level-0 candidates, then up to beam x children per level
    cand = [counts[0]] + [min(W, counts[l - 1]) * b for l in range(1, L)]
    # kernels per step: the read encode + the descent.  Grouped: max-children, bit packing
    # (with sign-bit reads and the caller's child count: the count's check instead) and
    # output, and per level count / 3 scan kernels / expand / select plus the scoring:
    # on CUDA cores 3 scan kernels / scatter / score; on the tensor cores (every level but
    # the last; the default) level 0 its item list and descent_tc_kernel, a later level the
    # parents' entry count / 3 scans / scatter, item count / 2 x 3 scans / write and
    # descent_tc_kernel.  One warp per read: one kernel.
    grouped = args.beam_grouped != 0 and dim % 1024 == 0 and dim <= 16384
    tc_levels = grouped and args.beam_grouped in (-1, 2)
    if not grouped:  # one warp per read
        per_step = 2
    elif args.beam_one == 1:  # every level in one cooperative launch
        per_step = 2
    elif args.beam_one == 2:  # the cooperative launch up to the leaf pairs, then a cooperative leaf kernel
        per_step = 3
    elif tc_levels and L > 1:
        per_step = 1 + 3 + 6 * L + 2 + 14 * (L - 2) + 5
    else:
        per_step = 1 + 3 + 11 * L
    res = dict(ms=ms, e2e_ms=e2e_ms, search_ms=float(np.median(beam_ms)), clocks=clk.summary(),
               launches=per_step * args.steps, refs=int(base[-1]), h2d=io["h2d"], d2h=io["d2h"], tree=tree,
               bundle=bundle, depth_mean=depth_mean, rows_per_read=int(sum(cand)), leaf_accuracy=leaf_acc,
               mean_len=float(np.mean(pool[0].len)), n_wide=n_wide, phases=phases, alt=alt,
               proto_bytes=n_wide * dim * 4 + (n_nodes - n_wide) * dim * 2)
    if not args.no_cpu_baseline:
        # q8 and out["r"] hold the last step's batch and result
        res["cpu"] = cpu_baseline_descent(cfg, pool[0], q8[:256].cpu().numpy(), proto, pn, ptr, idx,
                                          list(range(counts[0])))
        p_, s_, d_ = (x.cpu().numpy() for x in out["r"])
        res["sample_identical"] = all(
            d_[i] == len(wp) and list(p_[i, :len(wp)]) == wp and np.array_equal(s_[i, :len(wp)],
                                                                                np.array(ws, np.float32))
            for i, (wp, ws) in enumerate(res["cpu"].pop("paths")))
    return res


def descent_phases(ms, levels, grouped_tc=True, apart=False):
    """Per-level times (ms) of a one-launch descent from its phase clock: a level's
    phases end at its scoring; the select of a level is counted with the next.  With the
    last level apart (the default) the cooperative launch ends at that level's
    node-ordered pairs; leaf_kernel, a second cooperative launch timed with the
    call, scores them and takes the final beams."""
    names = ["setup"]
    for L in range(levels):
        tcl = grouped_tc and L < levels - 1
        if tcl and L == 0:
            names += ["count", "expand", "score_tc"]
        elif tcl:
            names += ["count", "expand", "parent_sums", "parent_scan", "scatter", "items", "score_tc"]
        elif apart:
            names += ["count", "expand", "node_sums", "node_scan", "scatter"]
        else:
            names += ["count", "expand", "node_sums", "node_scan", "scatter", "score_cuda"]
    names += ["handoff" if apart else "select_output"]
    if len(ms) != len(names):
        return {"raw_ms": ms}
    out = {"setup": ms[0]}
    per_level = [dict() for _ in range(levels)]
    i = 1
    for L in range(levels):
        tcl = grouped_tc and L < levels - 1
        n = 3 if (tcl and L == 0) else 7 if tcl else (5 if apart else 6)
        for nm in names[i:i + n]:
            per_level[L][nm] = per_level[L].get(nm, 0.0) + ms[i]
            i += 1
    out["levels"] = [{k: round(v, 4) for k, v in d.items()} for d in per_level]
    out[names[-1]] = ms[-1]
    out["total_cooperative"] = sum(ms)
    return out


def first_int16_row(proto, chunk=8192):
    """The smallest n such that every row of proto from n on fits int16."""
    import torch
    fits = torch.empty(proto.shape[0], dtype=torch.bool, device=proto.device)
    for i in range(0, proto.shape[0], chunk):
        fits[i:i + chunk] = proto[i:i + chunk].abs().amax(dim=1) <= 32767
    bad = torch.nonzero(~fits).flatten()
    return int(bad[-1]) + 1 if bad.numel() else 0


def cpu_baseline_descent(cfg, reads, q8, proto, pn, ptr, idx, roots, seconds=12.0):
    """The descent restated on the CPU (oracle beam_search, exact int64 dots,
    one core) for a bounded sample of the same reads, over a host copy of the
    same prototypes; also checks those reads' paths against the GPU's."""
    from oracle import oracle as O
    pn_h = proto_rows = None
    need = proto.numel() * 4
    if host_available_bytes() > 3 * need:
        proto_rows, how = proto.cpu().numpy(), "host copy"
    else:  # not enough host memory for a copy: the rows each step gathers are copied from the device
        proto_rows, how = _DeviceRows(proto), "rows gathered from device memory per step"
    pn_h = pn.cpu().numpy()
    done, t_total, paths = 0, 0.0, []
    while t_total < seconds and done < q8.shape[0]:
        t0 = time.time()
        paths += O.beam_search(q8[done:done + 8], proto_rows, ptr, idx, roots, cfg["levels"], cfg["beam"],
                               cfg["threshold"], O.SCORE_NORM, pn=pn_h)
        t_total += time.time() - t0
        done += min(8, q8.shape[0] - done)
    return dict(value=done / t_total, cores=1, done=done, rows=how, paths=paths)


def host_available_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


class _DeviceRows:
    """proto[nodes] for the CPU descent, copied from device memory on demand."""

    def __init__(self, t):
        self.t = t

    def __getitem__(self, nodes):
        import torch
        return self.t[torch.as_tensor(np.asarray(nodes), device=self.t.device)].cpu().numpy()


def oracle_database(cfg, threads):
    """Reference hypervectors for the reference arm, built on the CPU by the
    oracle from the same seeded workload as the GPU arm (no GPU library is
    loaded): leaf encodings (c2), or, for the bundled configurations, the exact
    sum of the same 8 noisy copies of each leaf (encode_copy_bundles: the
    leaf's encoding plus the k-mers each copy changes).  Rows are
    bit-identical to the GPU arm's database."""
    import hdc_synth as S
    from oracle import oracle as O
    tree = S.synth_tree(cfg["tree_seed"], cfg["n_leaves"])
    nr, dim = cfg["n_leaves"], cfg["dim"]
    if not cfg["copies"]:
        refs = O.encode_bundles(tree.buf, tree.off, tree.len, dim, cfg["kmer"], 1, threads).astype(np.int16)
        return tree, refs
    refs = np.empty((nr, dim), np.int16)
    chunk = 8192  # the GPU arm's chunks: copy seeds are per chunk
    for a in range(0, nr, chunk):
        b = min(nr, a + chunk)
        sub = S.Seqs(tree.buf, tree.off[a:b], tree.len[a:b])
        cp = S.synth_copies(cfg["copy_seed"] + a, sub, cfg["copies"], 0.01)
        refs[a:b] = O.encode_copy_bundles(sub, cp, cfg["copies"], dim, cfg["kmer"], threads)
    return tree, refs


def cpu_calls(cfg, refs, reads, first, n, threads, exact=False):
    """The reference CPU algorithm (oracle restatement: HVCache::compute per read,
    then brute-force cosine over every reference, top-k) on reads first ..
    first + n - 1 of `reads`, in calls of 2 x threads reads (two per thread).
    Returns (seconds, [scores, idx, cos, dot] or None)."""
    from oracle import oracle as O
    per_call = 2 * threads
    outs, t_total = [], 0.0
    for a in range(first, first + n, per_call):
        batch = [reads.get(j % len(reads)) for j in range(a, min(first + n, a + per_call))]
        t0 = time.time()
        r = O.classify(batch, refs, cfg["dim"], cfg["kmer"], cfg["topk"], O.SCORE_NORM, cfg["bipolar"], threads,
                       exact=exact)
        t_total += time.time() - t0
        outs.append(r)
    if not exact:
        return t_total, None
    return t_total, [np.concatenate([o[x] for o in outs]) for x in range(4)]


def cpu_baseline(cfg, refs, reads, gpu_out, min_reads=256, seconds=12.0, threads=None):
    """cpu_baseline leg of our arm: the oracle on the first reads of the GPU
    arm's own timed batch, against the same database (rows copied from the
    device), until both min_reads reads and `seconds` are done; the same reads'
    GPU results are compared with it (the parity sample)."""
    from oracle import oracle as O
    threads = threads or (os.cpu_count() or 1)
    O.ref_norms(refs, threads)  # once per database, outside the timed calls
    per_call = 2 * threads
    done, t_total, res = 0, 0.0, []
    limit = gpu_out[0].shape[0]
    while (done < min_reads or t_total < seconds) and done + per_call <= limit:
        dt, r = cpu_calls(cfg, refs, reads, done, per_call, threads, exact=True)
        t_total += dt
        done += per_call
        res.append(r)
    cs, ci, cc, cd = (np.concatenate([r[x] for r in res]) for x in range(4))
    gs, gi, gc, gd = (None if g is None else g[:done] for g in gpu_out)
    parity = {"reads": done, "from": "the first %d reads of the timed batch" % done,
              "topk_indices_identical": bool(np.array_equal(gi, ci)),
              "float_scores_identical": bool(np.array_equal(gs, cs)),
              "oracle": "oracle/hdc_oracle.c classify (HVCache::compute, int64 dots, FP64 cosine, "
                        "ties to the lower index)"}
    ok = parity["topk_indices_identical"] and parity["float_scores_identical"]
    if gd is not None:  # the search entry points also return each hit's exact dot and FP64 cosine
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = np.abs(gc - cc) / np.maximum(np.abs(cc), np.finfo(np.float64).tiny)
        parity["dots_identical"] = bool(np.array_equal(gd, cd))
        parity["cosine_fp64_max_rel_err"] = float(rel.max()) if rel.size else 0.0
        parity["cosine_fp64_bound"] = 1e-12
        ok = ok and parity["dots_identical"] and parity["cosine_fp64_max_rel_err"] <= 1e-12
    parity["identical"] = ok
    return done / t_total, threads, done, parity


def run_reference(args, cfg):
    """Reference arm: the reference CPU path on the host cores, per step a
    bounded sample (2 reads per core) of the GPU arm's own reads."""
    import hdc_synth as S
    threads = os.cpu_count() or 1
    t0 = time.time()
    tree, refs = oracle_database(cfg, threads)
    log("oracle database built in %.1f s" % (time.time() - t0))
    from oracle import oracle as O
    reads = make_reads(S, tree, cfg, 4096, cfg["read_seed"])  # the GPU arm's first reads
    O.ref_norms(refs, threads)  # once per database, outside the timed calls
    vals, per_call = [], 2 * threads
    for i in range(args.warmup + args.steps):
        dt, _ = cpu_calls(cfg, refs, reads, (i * per_call) % len(reads), per_call, threads)
        if i >= args.warmup:
            vals.append(per_call / dt)
    return float(np.median(vals)), threads, per_call


def batching_line(args, b, refs_host, pk):
    """The batching form measured inside the c3 run (same database): reads/s
    resident and end to end, its search's roofline, the autotuned schedule and
    the oracle's parity sample on the first reads of its batch."""
    cfg = b["cfg"]
    B = args.batch
    flops = 2.0 * cfg["dim"] * b["refs"] * b["limbs"] * B
    achieved = flops / (b["search_ms"] / 1e3) / 1e12
    out = {"workload": "c4 reads on this database: log-normal lengths (median %d bp, sigma %.1f, %d-%d bp), %d%% "
                       "with %d%% sub:ins:del 3:1:1, top-%d, CUDA-graph encode -> search -> top-k" % (
                           cfg["read_len"], cfg["sigma"], cfg["min_read"], cfg["max_read"], 100 * cfg["mixed_frac"],
                           100 * cfg["mixed_rate"], cfg["topk"]),
           "value": B / (b["ms"] / 1e3), "unit": "reads/s", "batch_reads": B, "ms_per_step": b["ms"],
           "e2e": {"value": B / (b["e2e_ms"] / 1e3), "unit": "reads/s", "h2d_bytes_per_step": b["h2d"],
                   "d2h_bytes_per_step": b["d2h"]},
           "search_roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"],
                               "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"]},
           "autotuned_schedule": b["tuned"], "mean_read_len": b["mean_len"], "top1_accuracy": b["top1_accuracy"],
           "gpu_launches": b["launches"], "clocks": b["clocks"]}
    if refs_host is not None:
        _, _, _, parity = cpu_baseline(cfg, refs_host, b["reads"], b["gpu_first"], min_reads=128, seconds=0.0)
        out["parity_sample"] = parity
    return out


def descent_line(args, cfg, r, metric, workload):
    """The JSON line of the hierarchical-descent form."""
    pk, src = peaks()
    B, dim = args.batch, cfg["dim"]
    # grouped descent: every prototype row is a candidate at its own rank's level only, so a
    # call reads each at most once, plus each level's packed +1/-1 reads
    algo_bytes = r["proto_bytes"] + cfg["levels"] * B * dim / 8
    split = r["n_wide"] < r["refs"]
    achieved = algo_bytes / (r["search_ms"] / 1e3) / 1e9
    bundle_bytes = sum(x["bytes"] for x in r["bundle"])
    bundle_ms = sum(x["ms"] for x in r["bundle"])
    line = {
        "metric": metric, "value": B / (r["ms"] / 1e3), "unit": "reads/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "%s x %s prototypes, exact int64 dots, FP64 scores" % (
            "+1/-1 reads as sign bits" if split else "int8 +1/-1 reads",
            "int32 (ranks above) / int16 (nodes %d on)" % r["n_wide"] if split else "int32"),
        "data": "synthetic (seeded 6-rank tree, see bench.py)",
        "config": {"workload": workload, "form": "descent", "batch_reads": B, "nodes": r["refs"],
                   "mean_read_len": r["mean_len"], "mean_depth": r["depth_mean"],
                   "leaf_accuracy": r["leaf_accuracy"],
                   "int16_rows_from_node": r["n_wide"],
                   "l2": "inputs larger than L2: %.1f GB of prototypes, the lower ranks gathered from HBM "
                         "every step" % (r["proto_bytes"] / 1e9)},
        "e2e": {"value": B / (r["e2e_ms"] / 1e3), "unit": "reads/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": TRAFFIC_DESCENT.get((B, split)),
                     "traffic_source": "ncu DRAM bytes of the scoring launches of one full-size call "
                                       "(descent_tc_kernel x 5 + score_kernel; measured at 38,912 reads; "
                                       "null at other batch sizes)",
                     "peak_source": "%s HBM copy bandwidth (MEASURED_PEAKS.json)" % src,
                     "kernel": "grouped descent (hdc_beam_search%s, %s: per level count/expand/select; "
                               "levels above the leaves scored on the tensor cores, the leaves on the CUDA "
                               "cores), timed as one call; algorithmic bytes = the %.1f GB "
                               "of prototypes once + %d levels of packed reads; the tensor-core levels are "
                               "bound by their producers' conversions, the leaf level by HBM "
                               "(%d candidate rows per read)" % (
                                   "_split" if split else "",
                                   "descent_one_kernel, every level in one cooperative launch" if args.beam_one == 1
                                   else "kernels per level" if args.beam_one == 0
                                   else "descent_one_kernel, every level in one cooperative launch up to the "
                                        "leaf pairs sorted by node, then leaf_kernel (cooperative) scoring them "
                                        "and taking the final beams", r["proto_bytes"] / 1e9,
                                   cfg["levels"],
                                   r["rows_per_read"])},
        "propagate_bundle": {"kernel": "bundle_kernel (internal prototypes = int32 sums of children)",
                             "ms": bundle_ms, "gb_per_s": bundle_bytes / (bundle_ms / 1e3) / 1e9,
                             "frac_of_hbm": bundle_bytes / (bundle_ms / 1e3) / 1e9 / pk["hbm_gbs"],
                             "per_rank": r["bundle"]},
        "clocks": r["clocks"], "gpu_launches": r["launches"],
    }
    if r.get("alt"):
        line["kernels_per_level_form"] = r["alt"]
    if r.get("phases"):
        line["descent_phases_ms"] = r["phases"]
    if "sample_identical" in r:
        line["paths_identical_to_oracle"] = {"reads": r["cpu"]["done"], "identical": r["sample_identical"]}
    if "cpu" in r:
        line["cpu_baseline"] = {"value": r["cpu"]["value"], "unit": "reads/s", "cores": r["cpu"]["cores"],
                                "kind": "port", "sample": "%d reads of the same batch: the descent restated "
                                                          "(oracle, exact int64 dots) over the same prototypes "
                                                          "(%s); encode excluded" % (r["cpu"]["done"],
                                                                                     r["cpu"]["rows"])}
    return line


_DESCENT = {}


def run_reference_descent(args, cfg):
    """Reference arm of the descent: prototypes built on the CPU (the oracle's
    encoder + int32 sums of children), then per step a bounded sample of reads
    encoded and descended by the oracle on every host core (forked workers
    sharing the prototypes; no GPU in this process)."""
    import multiprocessing as mp
    import hdc_synth as S
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    t0 = time.time()
    tree = S.synth_tree(cfg["tree_seed"], cfg["n_leaves"])
    b, base, counts, ptr, idx = S.synth_tree_csr(cfg["n_leaves"])
    dim = cfg["dim"]
    proto = np.empty((int(base[-1]), dim), np.int32)
    leaf0 = int(base[5])
    for a in range(0, cfg["n_leaves"], 65536):
        e = min(cfg["n_leaves"], a + 65536)
        proto[leaf0 + a:leaf0 + e] = O.encode_bundles(tree.buf, tree.off[a:e], tree.len[a:e], dim, cfg["kmer"], 1,
                                                      threads)
    for r_ in range(4, -1, -1):  # children of a parent are consecutive rows of the rank below
        lo, hi = int(base[r_]), int(base[r_ + 1])
        first = idx[ptr[lo:hi]]
        proto[lo:hi] = np.add.reduceat(proto[int(base[r_ + 1]):int(base[r_ + 2])], first - int(base[r_ + 1]), axis=0)
    pn = np.concatenate([(proto[a:a + 4096].astype(np.int64) ** 2).sum(1) for a in range(0, len(proto), 4096)])
    log("CPU prototypes built in %.1f s" % (time.time() - t0))
    _DESCENT.update(proto=proto, pn=pn, ptr=ptr, idx=idx, roots=list(range(counts[0])), levels=cfg["levels"],
                    beam=cfg["beam"], threshold=cfg["threshold"])
    reads = make_reads(S, tree, cfg, 16 * threads * 8, cfg["read_seed"])  # the GPU arm's first reads
    vals, done = [], 0
    with mp.get_context("fork").Pool(threads) as pool:
        for i in range(args.warmup + args.steps):
            n = 2 * threads if i < args.warmup else 8 * threads
            seqs = [reads.get(j % len(reads)) for j in range(i * n, (i + 1) * n)]
            t1 = time.time()
            q, _ = O.encode(seqs, dim, cfg["kmer"], "bipolar", threads)
            done_n = sum(pool.map(_descent_worker_q, [q[j:j + 2] for j in range(0, n, 2)]))
            dt = time.time() - t1
            if i >= args.warmup:
                vals.append(done_n / dt)
                done = done_n
    return float(np.median(vals)), threads, done


def _descent_worker_q(q):
    from oracle import oracle as O
    d = _DESCENT
    return len(O.beam_search(q, d["proto"], d["ptr"], d["idx"], d["roots"], d["levels"], d["beam"], d["threshold"],
                             O.SCORE_NORM, pn=d["pn"]))


def _event_ms(fn, reps=5):
    """Median CUDA-event time (ms) of fn() on the current stream, after one warm-up call."""
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = []
    for _ in range(reps):
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return float(np.median(out))


def fasta_bytes(n_records, read_len, line=60, seed=0):
    """A FASTA file of n_records random reads (names ">r" + 9 digits) in lines of `line` bases."""
    rng = np.random.default_rng(seed)
    bases = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, (n_records, read_len))]
    nl = (read_len + line - 1) // line
    body = np.full((n_records, read_len + nl), ord("\n"), np.uint8)
    for j in range(nl):
        a, b = j * line, min(read_len, (j + 1) * line)
        body[:, a + j:b + j] = bases[:, a:b]
    ids = np.arange(n_records)
    name = np.empty((n_records, 11), np.uint8)
    name[:, 0] = ord(">")
    name[:, 1] = ord("r")
    for p in range(9):
        name[:, 10 - p] = ord("0") + (ids // 10 ** p) % 10
    return np.concatenate([name, np.full((n_records, 1), ord("\n"), np.uint8), body], axis=1).reshape(-1)


def run_aux(args):
    """Kernels beside the headline path, at sizes above L2, each timed alone with CUDA events
    (median of 5 after a warm-up): FASTA ingest, 2-bit packing, read encode from ASCII and from
    packed words, windowed similarity.  One JSON line with each kernel's time and achieved
    bandwidth against the measured HBM peak."""
    import torch
    import hdc_gb300 as H
    pk, src = peaks()
    hbm = pk["hbm_gbs"]
    dev = torch.device("cuda", 0)
    out = {}
    scale = args.aux_scale
    # FASTA ingest: 3,000,000 records of 250 bp in 60-column lines (times the scale)
    n_fa = max(40000, int(3000000 * scale))
    data = fasta_bytes(n_fa, 250)
    d = torch.from_numpy(data).to(dev)
    ctx = H.Context(10240, 10, 250, 10)
    ms = _event_ms(lambda: ctx.fasta_parse(d, n_fa + 1))
    seq_bytes, so, sl, _, _, n_rec = ctx.fasta_parse(d, n_fa + 1)
    out["fasta_parse"] = {"input_bytes": int(d.numel()), "records": int(n_rec), "ms": ms,
                          "input_gb_per_s": d.numel() / (ms / 1e3) / 1e9,
                          "note": "8 KB tiles: the input read twice, the sequences written once, a few words "
                                  "per tile and per record"}
    # 2-bit packing of the parsed sequence bytes (read 1 byte, write 1/4 byte per base)
    n_seq = int(so[-1] + sl[-1])
    words = ctx.pack_2bit(seq_bytes, n_seq)
    ms = _event_ms(lambda: ctx.pack_2bit(seq_bytes, n_seq))
    moved = n_seq + 4 * ((n_seq + 15) // 16)
    out["pack_2bit"] = {"bases": n_seq, "ms": ms, "gb_per_s": moved / (ms / 1e3) / 1e9,
                        "frac_of_hbm": moved / (ms / 1e3) / 1e9 / hbm}
    # read encode, c3 shape (38,912 reads of 250 bp, D = 10,240, k = 10, +1/-1 fp16 rows), from
    # ASCII and from packed words
    B = min(38912, n_fa)
    offs, lens = so[:B], sl[:B]
    q = torch.empty((B, 10240), dtype=torch.float16, device=dev)
    t_ascii = _event_ms(lambda: ctx.encode_segments(seq_bytes, offs, lens, q, H.OUT_BIPOLAR_F16, 250))
    a = q.clone()
    t_packed = _event_ms(lambda: ctx.encode_packed(words, offs, lens, q, H.OUT_BIPOLAR_F16, 250))
    torch.cuda.synchronize()
    out["encode_reads"] = {"reads": B, "ascii_ms": t_ascii, "packed_ms": t_packed,
                           "identical": bool(torch.equal(a, q)),
                           "reads_per_s_ascii": B / (t_ascii / 1e3), "reads_per_s_packed": B / (t_packed / 1e3),
                           "bound": "integer/logic pipe (bundling), not bytes: 250 B of ASCII per read in"}
    del d, seq_bytes, words, q, a
    # windowed similarity (HVCache::similarity batched): 4,096 queries of 150 bp x 16 references of
    # 1,500 bp each (135 windows), D = 8,192, k = 8
    sctx = H.Context(8192, 8, 150, 10)
    tree = H.synth_tree(21, 2000)
    reads = H.synth_reads(22, tree, 4096, 150, subst=0.01)
    wins_off, ref_rows, whole = [], [0], []
    for i in range(len(tree)):
        o, n = int(tree.off[i]), int(tree.len[i])
        xs = list(range(0, n - 150, 10))
        wins_off += [o + x for x in xs]
        ref_rows.append(len(wins_off))
        whole.append(0)
    d_tree = torch.from_numpy(tree.buf).to(dev)
    rows = torch.empty((len(wins_off), 8192), dtype=torch.int16, device=dev)
    sctx.encode_segments(d_tree, torch.tensor(wins_off, dtype=torch.int64, device=dev),
                         torch.full((len(wins_off),), 150, dtype=torch.int32, device=dev), rows, H.OUT_I16, 150)
    qv = torch.empty((4096, 8192), dtype=torch.int16, device=dev)
    sctx.encode_segments(torch.from_numpy(reads.buf).to(dev), torch.from_numpy(reads.off).to(dev),
                         torch.from_numpy(reads.len).to(dev), qv, H.OUT_I16, 150)
    qn, rn = sctx.norms(qv), sctx.norms(rows)
    g = np.random.default_rng(5)
    pq = np.repeat(np.arange(4096), 16).astype(np.int32)
    pr = (np.asarray(reads.label)[pq] + g.integers(-8, 8, pq.size)).clip(0, len(tree) - 1).astype(np.int32)
    d_rr = torch.tensor(ref_rows, dtype=torch.int64, device=dev)
    d_pq, d_pr = torch.from_numpy(pq).to(dev), torch.from_numpy(pr).to(dev)
    ms = _event_ms(lambda: sctx.similarity(qv, qn, rows, rn, d_rr, None, d_pq, d_pr))
    n_pairs = pq.size
    row_bytes = float(np.sum(np.diff(ref_rows)[pr])) * 8192 * 2
    out["similarity"] = {"pairs": int(n_pairs), "window_rows_read": int(np.sum(np.diff(ref_rows)[pr])), "ms": ms,
                         "row_gb_per_s": row_bytes / (ms / 1e3) / 1e9,
                         "unique_row_bytes": int(rows.numel() * 2),
                         "note": "row bytes of every pair (rows shared by pairs come from L2)"}
    del rows, qv
    # propagate-children's greedy representatives and identify's descent on a tree of the C1
    # shape: 2,000 leaves of 1,400-1,600 bp (times the scale), D = 8,192, k = 8
    n_leaves = max(200, int(2000 * scale))
    tree = H.synth_tree(23, n_leaves)
    d_tree = torch.from_numpy(tree.buf).to(dev)
    hv = torch.empty((n_leaves, 8192), dtype=torch.int16, device=dev)
    sctx.encode_segments(d_tree, torch.from_numpy(tree.off).to(dev), torch.from_numpy(tree.len).to(dev), hv,
                         H.OUT_I16, tree.max_len())
    hn = sctx.norms(hv)
    b, base, counts, cptr, cidx = H.synth_tree_csr(n_leaves)
    groups = []  # every internal node with its descendant leaves, in order
    for r in range(1, 6):
        span = b ** (6 - r)
        groups += [list(range(j * span, min(n_leaves, (j + 1) * span))) for j in range(counts[r - 1])]
    cand_ptr = np.zeros(len(groups) + 1, np.int64)
    cand_ptr[1:] = np.cumsum([len(x) for x in groups])
    cand_idx = np.array([x for grp in groups for x in grp], np.int32)
    t = lambda a: torch.from_numpy(a).to(dev)
    gp, gi, rp, ri = t(cand_ptr), t(cand_idx), t(np.zeros(len(groups) + 1, np.int64)), t(np.zeros(1, np.int32))
    ms = _event_ms(lambda: sctx.propagate_greedy(hv, hn, gp, gi, rp, ri, 0.75))
    sel, _ = sctx.propagate_greedy(hv, hn, gp, gi, rp, ri, 0.75)
    out["propagate_greedy"] = {"parents": len(groups), "candidates": int(cand_idx.size),
                               "selected": int(sel.sum().item()), "ms": ms,
                               "form": "scored: pair scores in bulk (tiled), then each parent's decisions in "
                                       "order from running maxima"}
    # identify: a leaf's similarity rows are its windows (135 of 150 bp, step 10); an internal
    # node's are the first 20 windows of its first descendant leaf
    row_off, node_rows = [], [0]
    for node in range(int(base[-1])):
        rank = int(np.searchsorted(base, node, side="right")) - 1
        leaf = (node - int(base[rank])) * b ** (5 - rank)
        o, n = int(tree.off[leaf]), int(tree.len[leaf])
        xs = list(range(0, n - 150, 10))
        if rank < 5:
            xs = xs[:20]
        row_off += [o + x for x in xs]
        node_rows.append(len(row_off))
    rows = torch.empty((len(row_off), 8192), dtype=torch.int16, device=dev)
    sctx.encode_segments(d_tree, torch.tensor(row_off, dtype=torch.int64, device=dev),
                         torch.full((len(row_off),), 150, dtype=torch.int32, device=dev), rows, H.OUT_I16, 150)
    rn = sctx.norms(rows)
    reads = H.synth_reads(24, tree, 4096, 150, subst=0.01)
    qv = torch.empty((4096, 8192), dtype=torch.int16, device=dev)
    sctx.encode_segments(torch.from_numpy(reads.buf).to(dev), torch.from_numpy(reads.off).to(dev),
                         torch.from_numpy(reads.len).to(dev), qv, H.OUT_I16, 150)
    qn = sctx.norms(qv)
    d_nr, d_cp, d_ci = t(np.array(node_rows, np.int64)), t(cptr), t(cidx)
    d_roots = torch.arange(counts[0], dtype=torch.int32, device=dev)
    # threshold -2 (below every NORM score): every read descends all six ranks
    ms = _event_ms(lambda: sctx.identify(qv, qn, rows, rn, d_nr, d_cp, d_ci, d_roots, 6, 5, -2.0))
    path, _, depth, _ = sctx.identify(qv, qn, rows, rn, d_nr, d_cp, d_ci, d_roots, 6, 5, -2.0)
    out["identify"] = {"reads": 4096, "nodes": int(base[-1]), "similarity_rows": len(row_off),
                       "row_bytes": len(row_off) * 8192 * 2, "ms": ms, "reads_per_s": 4096 / (ms / 1e3),
                       "mean_depth": float(depth.float().mean().item()),
                       "bound": "gathers of each candidate node's rows (one CTA per read)"}
    line = {"metric": "auxiliary kernels (ms, GB/s)", "unit": "ms", "n_gpus": 1, "higher_is_better": False,
            "data": "synthetic", "config": {"workload": "aux: FASTA ingest, 2-bit packing, read encode, "
                                                         "windowed similarity, propagate greedy, identify",
                                            "scale": scale},
            "peak_hbm_gbs": hbm, "peak_source": "%s (MEASURED_PEAKS.json)" % src, "kernels": out}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c3", choices=sorted(CONFIGS) + ["aux"])
    ap.add_argument("--form", default="", choices=["", "plain", "tc", "pipe", "descent"],
                    help="default: tc for c3, pipe for c4, plain for c2, descent for c5")
    ap.add_argument("--batch", type=int, default=0,
                    help="reads per step; 0 = 2 x SMs x 128, whole waves of 128-query tensor-core tiles")
    ap.add_argument("--plain-batch", type=int, default=4096)
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain form beside the tc form")
    ap.add_argument("--no-batching", action="store_true",
                    help="c3: skip the batching form (c4 reads through the pipeline) on the same database")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--refs", type=int, default=0, help="override the number of references (small profiling cases)")
    ap.add_argument("--topk", type=int, default=0, help="override k of the top-k search (0: the workload's)")
    ap.add_argument("--tc-group", type=int, default=0, help="tensor-core search: query tiles per group (0: library default)")
    ap.add_argument("--tc-cluster", type=int, default=0, help="tensor-core search: CTAs sharing reference blocks (0: default)")
    ap.add_argument("--beam-grouped", type=int, default=-1,
                    help="descent: 1 reads grouped by candidate node, 0 one warp per read (-1: default)")
    ap.add_argument("--beam-one", type=int, default=-1,
                    help="descent: 1 every level in one launch, 2 one launch up to the leaf pairs + a leaf launch, "
                         "0 kernels per level (-1: the library default, 2)")
    ap.add_argument("--score-mode", default="norm", choices=["norm", "cos", "dot"],
                    help="score of the top-k search (default the reference's NORM scale; the CPU legs need it)")
    ap.add_argument("--aux-scale", type=float, default=1.0,
                    help="aux: sizes of the FASTA and tree cases times this (small profiling cases)")
    ap.add_argument("--proto-int32", action="store_true",
                    help="descent: every prototype row int32 (default: int16 rows from the first node whose rows fit)")
    args = ap.parse_args()
    if args.beam_one < 0:  # the library's automatic descent form: two cooperative launches
        args.beam_one = 2
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.config == "aux":  # kernels beside the headline path, timed one by one
        if int(os.environ.get("WORLD_SIZE", "1")) == 1 and args.impl == "ours":
            run_aux(args)
        return
    cfg = dict(CONFIGS[args.config])
    if not args.form:
        args.form = {"c1": "plain", "c2": "plain", "c3": "tc", "c4": "pipe", "c5": "descent"}[args.config]
    if args.refs:
        cfg["n_leaves"] = args.refs
    if args.topk:
        cfg["topk"] = args.topk
    if args.score_mode != "norm":
        if not args.no_cpu_baseline or args.impl == "reference":
            raise SystemExit("--score-mode other than norm needs --no-cpu-baseline (the oracle legs rank by NORM)")
        cfg["score_mode"] = args.score_mode
    if cfg.get("sigma"):
        reads_desc = "log-normal reads (median %d bp, sigma %.1f, %d-%d bp, %d%% with %d%% sub:ins:del 3:1:1)" % (
            cfg["read_len"], cfg["sigma"], cfg["min_read"], cfg["max_read"], 100 * cfg["mixed_frac"],
            100 * cfg["mixed_rate"])
        workload = "%s: %d refs D=%d k=%d, %s, top-%d" % (args.config, cfg["n_leaves"], cfg["dim"], cfg["kmer"],
                                                         reads_desc, cfg["topk"])
    else:
        workload = "%s: %d refs D=%d k=%d, %d bp reads, top-%d" % (args.config, cfg["n_leaves"], cfg["dim"], cfg["kmer"],
                                                                   cfg["read_len"], cfg["topk"])
    metric = "reads/s encode+top-%d search" % cfg["topk"]
    if args.form == "descent":
        metric = "reads/s encode+hierarchical descent (top-%d per rank, %d ranks, root to leaf)" % (cfg["beam"],
                                                                                                  cfg["levels"])
        workload = "%s: %d leaves + internal prototypes D=%d k=%d, %s" % (
            args.config, cfg["n_leaves"], cfg["dim"], cfg["kmer"], reads_desc)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 or args.gpus > 1:
        # single-GPU library: the tensor-core search's multicast loads stay within one GPU's memory
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"impl": args.impl, "metric": metric, "unit": "reads/s", "n_gpus": args.gpus,
                              "unavailable": "single-GPU library: every form runs on one GPU (reads are "
                                             "independent; run one process per GPU as separate replicas)"}),
                  flush=True)
        return
    if args.impl == "reference" and args.form == "descent":
        v, threads, done = run_reference_descent(args, cfg)
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "reads/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "int64",
                "data": "synthetic", "config": {"workload": workload},
                "cpu_baseline": {"value": v, "unit": "reads/s", "cores": threads, "kind": "port",
                                 "sample": "%d reads per step (HVCache::compute restated to +1/-1, then the "
                                           "beam descent restated with exact int64 dots); prototypes built on "
                                           "the CPU" % done},
                "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        v, threads, done = run_reference(args, cfg)
        line = {"impl": "reference", "metric": metric, "value": v, "unit": "reads/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "int64",
                "data": "synthetic", "config": {"workload": workload},
                "cpu_baseline": {"value": v, "unit": "reads/s", "cores": threads, "kind": "port",
                                 "sample": "%d reads per step, 2 per core, from the GPU arm's own reads "
                                           "(HVCache::compute restated + brute-force int64 cosine over all %d "
                                           "references); database rows built on the CPU from the same workload%s; "
                                           "%s" % (done, cfg["n_leaves"], " (sums of the same 8 noisy copies)"
                                                   if cfg["copies"] else "", PORT_NOTE)},
                "e2e": {"value": v, "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    if args.batch <= 0 and cfg.get("batch"):
        args.batch = cfg["batch"]
    if args.batch <= 0:
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        args.batch = 2 * sms * 128
    if args.form == "descent":
        r = run_descent(args, cfg)
        print(json.dumps(descent_line(args, cfg, r, metric, workload)), flush=True)
        return
    r = run_ours(args, cfg)
    pk, src = peaks()
    B = args.batch
    value = B / (r["ms"] / 1e3)
    dim, nr = cfg["dim"], r["refs"]
    if args.form in ("tc", "pipe"):
        # tensor work per read: one fp16 MMA pass per limb, 2*D*R*limbs flops
        flops = 2.0 * dim * nr * r["limbs"] * B
        achieved = flops / (r["search_ms"] / 1e3) / 1e12
        tile_pairs = ((B + 127) // 128) * (((nr + 255) // 256) * 2)
        roof = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": TRAFFIC_PER_TILE_PAIR_TC * tile_pairs,
                "traffic_source": "ncu DRAM bytes of the two search launches of a full-size c3 call, per "
                                  "128x128 tile pair, times this call's %d pairs (query tiles re-read for every "
                                  "reference tile, half of them through L2)" % tile_pairs,
                "peak_source": "%s dense bf16/fp16 burst (MEASURED_PEAKS.json)" % src,
                "kernel": "tc_search_kernel (clusters of 4 + pair remainder) + merge, %d fp16 limbs; "
                          "algorithmic 2*D*R*limbs per read" % r["limbs"]}
        dtype = "fp16 integer limbs, fp32 accumulators (exact int64 dots), FP64 scores"
    else:
        flops = 2.0 * dim * nr * B
        achieved = flops / (r["search_ms"] / 1e3) / 1e12
        sm_mhz = r["clocks"].get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        roof = {"bound": "fp32-pipe", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": None,
                "peak_source": "152 SMs x 128 FFMA x 2 x median SM clock",
                "kernel": "plain_kernel + merge on CUDA cores; algorithmic 2*D*R per read"}
        dtype = "int16 (exact integer dots on the fp32 pipe), FP64 scores"
    line = {
        "metric": metric, "value": value, "unit": "reads/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded 6-rank tree, see bench.py)",
        "config": {"workload": workload, "form": args.form, "batch_reads": B,
                   "l2": "inputs larger than L2: %.0f MB reference database streamed every step" %
                         (nr * dim * 2 * max(1, r["limbs"]) / 1e6)},
        "e2e": {"value": B / (r["e2e_ms"] / 1e3), "unit": "reads/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "roofline": roof, "clocks": r["clocks"], "gpu_launches": r["launches"],
    }
    if "top1_accuracy" in r:
        line["config"]["top1_accuracy"] = r["top1_accuracy"]  # top hit = the read's source leaf
    if "known_answer" in r:
        line["known_answer"] = r["known_answer"]
    if "tuned" in r:
        line["config"]["autotuned_schedule"] = r["tuned"]
        line["config"]["mean_read_len"] = r["mean_len"]
    if "plain" in r:
        line["plain_form"] = {"value": r["plain"]["value"], "unit": "reads/s", "batch_reads": r["plain"]["batch"],
                              "speedup_tc_over_plain": value / r["plain"]["value"],
                              "labels_identical": r["labels_identical_to_plain"]}
    if "tc_form" in r:
        t = r["tc_form"]
        line["tc_form"] = {"value": t["value"], "unit": "reads/s", "batch_reads": B,
                           "speedup_tc_over_plain": t["value"] / value, "limbs": t["limbs"],
                           "limb_base": 1 << t["limb_bits"], "labels_identical": t["labels_identical"],
                           "scores_identical": t["scores_identical"],
                           "note": "the same count-valued reads as fp16 queries on the tensor cores, the "
                                   "database's limbs sized for the largest count (exact)"}
        if "tc_known_answer" in r:
            line["tc_form"]["known_answer"] = r["tc_known_answer"]
    if not args.no_cpu_baseline:
        v, threads, done, parity = cpu_baseline(cfg, r["refs_host"], r["reads"], r["gpu_first"])
        line["cpu_baseline"] = {"value": v, "unit": "reads/s", "cores": threads, "kind": "port",
                                "sample": "the first %d reads of the timed batch, %d per call (encode + "
                                          "brute-force top-%d against all %d references, the database rows copied "
                                          "from the device); %s" % (done, 2 * threads, cfg["topk"], nr, PORT_NOTE)}
        line["parity_sample"] = parity
    if "batching" in r:
        line["batching_form"] = batching_line(args, r["batching"], r.get("refs_host"), pk)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
