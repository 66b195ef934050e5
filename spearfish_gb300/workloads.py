"""Seeded synthetic workloads in the shapes the alignment stage is benchmarked on.

The error model restates spearfish's read simulator (crates/spearfish-cli/src/sim.rs:59-99):
each base is deleted, substituted or kept, then an insertion may follow it; indel
probabilities are raised inside homopolymer runs (length >= 3) by `hp_bias` and scaled down
elsewhere so the mean rate stays as requested; insertions inside runs extend the run.  Random
draws come from numpy's PCG64 seeded per workload (the reference's SplitMix64 streams are
not reproduced: no output depends on them).

Workloads (sizes as the benchmark configurations state them):
  c1  Myers: 10,000 pairs, query uniform ACGT of 1,000 bases; target = query with 8%
      errors (sub:ins:del = 2:1:1), plus 50 random bases on each side; Infix.
  c2  banded affine with traceback: 20,000 pairs, query 2,000 bases; target = query with
      10% ONT-like errors -- indel-heavy (30% substitutions, 70% indels), deletions 40% of
      indel sites, indels raised 4x inside homopolymers; band 128, Affine{2,4,4,2}, Global.
  c3  uneven batch: 100,000 pairs, query length log-normal (median 1,200, sigma 0.8)
      clipped to 200..20,000; error rate uniform 5-12% with c2's profile; per pair a Myers
      Infix job (target + 50-base flanks) and a banded affine Global job with band
      clamp(32 * ceil(0.1 * L / 32), 64, 512).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Profile:
    sub: float
    ins: float
    dele: float
    hp_bias: float


UNIFORM_211 = Profile(0.50, 0.25, 0.25, 1.0)  # c1: sub:ins:del = 2:1:1
ONT_INDEL = Profile(0.30, 0.42, 0.28, 4.0)    # c2/c3: indel-heavy, del 40% of indels
HIFI = Profile(0.20, 0.40, 0.40, 10.0)        # sim.rs:38-45 `hifi`


def homopolymer_mask(seq: np.ndarray) -> np.ndarray:
    """sim.rs:60-72: base i lies in a run of >= 3 equal bases."""
    n = seq.size
    if n == 0:
        return np.zeros(0, dtype=bool)
    starts = np.concatenate([[0], np.flatnonzero(np.diff(seq) != 0) + 1])
    lens = np.diff(np.concatenate([starts, [n]]))
    return np.repeat(lens >= 3, lens)


def simulate(orig: np.ndarray, rate: float, p: Profile, rng: np.random.Generator) -> np.ndarray:
    """sim.rs:59-99 `simulate`, one pass of numpy draws per base."""
    n = orig.size
    hp = homopolymer_mask(orig)
    f_hp = float(hp.mean()) if n else 0.0
    scale = 1.0 / (1.0 - f_hp + p.hp_bias * f_hp)
    p_sub, p_ins, p_del = rate * p.sub, rate * p.ins, rate * p.dele
    bias = scale * np.where(hp, p.hp_bias, 1.0)
    r = rng.random(n)
    dele = r < p_del * bias
    subs = ~dele & (r < p_del * bias + p_sub)
    base = orig.copy()
    base[subs] = (orig[subs] + rng.integers(1, 4, int(subs.sum()), dtype=np.uint8)) & 3
    keep = ~dele
    ins = rng.random(n) < p_ins * bias
    ins_base = np.where(hp, orig, rng.integers(0, 4, n, dtype=np.uint8)).astype(np.uint8)
    counts = keep.astype(np.int64) + ins
    out = np.empty(int(counts.sum()), dtype=np.uint8)
    at = np.cumsum(counts) - counts
    out[at[keep]] = base[keep]
    out[(at + keep)[ins]] = ins_base[ins]
    return out


@dataclass
class Pairs:
    """Pairs as one pool of byte codes: pattern q at pool[p_off[q]:+m[q]], text likewise."""
    pool: np.ndarray
    p_off: np.ndarray
    m: np.ndarray
    t_off: np.ndarray
    n: np.ndarray
    band: np.ndarray      # per pair (affine)
    name: str

    def __len__(self):
        return int(self.m.size)

    def pattern(self, q: int) -> np.ndarray:
        return self.pool[self.p_off[q]:self.p_off[q] + self.m[q]]

    def text(self, q: int) -> np.ndarray:
        return self.pool[self.t_off[q]:self.t_off[q] + self.n[q]]

    def subset(self, idx) -> "Pairs":
        idx = np.asarray(idx)
        parts, p_off, t_off = [], [], []
        at = 0
        for q in idx:
            p, t = self.pattern(int(q)), self.text(int(q))
            p_off.append(at)
            parts.append(p)
            at += p.size
            t_off.append(at)
            parts.append(t)
            at += t.size
        pool = np.concatenate(parts) if parts else np.zeros(1, np.uint8)
        return Pairs(pool, np.array(p_off, np.uint64), self.m[idx].copy(),
                     np.array(t_off, np.uint64), self.n[idx].copy(), self.band[idx].copy(),
                     self.name)


def _assemble(ps, ts, bands, name) -> Pairs:
    m = np.array([p.size for p in ps], dtype=np.uint32)
    n = np.array([t.size for t in ts], dtype=np.uint32)
    inter = [x for pair in zip(ps, ts) for x in pair]
    sizes = np.array([x.size for x in inter], dtype=np.uint64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    pool = np.concatenate(inter) if inter else np.zeros(1, np.uint8)
    return Pairs(pool, offs[0::2].copy(), m, offs[1::2].copy(), n,
                 np.asarray(bands, dtype=np.uint64), name)


def config1(pairs: int = 10_000, seed: int = 1) -> Pairs:
    rng = np.random.default_rng(seed)
    ps, ts = [], []
    for _ in range(pairs):
        q = rng.integers(0, 4, 1000, dtype=np.uint8)
        t = simulate(q, 0.08, UNIFORM_211, rng)
        fl = rng.integers(0, 4, 100, dtype=np.uint8)
        ps.append(q)
        ts.append(np.concatenate([fl[:50], t, fl[50:]]))
    return _assemble(ps, ts, np.zeros(pairs), "c1")


def decoys(w: Pairs, seed: int = 11) -> Pairs:
    """w's patterns against unrelated texts of the same lengths: the candidates a tie-break's
    capped Global or Prefix distance call rejects."""
    rng = np.random.default_rng(seed)
    ps = [w.pattern(q) for q in range(len(w))]
    ts = [rng.integers(0, 4, int(w.n[q]), dtype=np.uint8) for q in range(len(w))]
    return _assemble(ps, ts, w.band, w.name + "-decoys")


def config2(pairs: int = 20_000, seed: int = 2, m: int = 2000, band: int = 128) -> Pairs:
    rng = np.random.default_rng(seed)
    ps, ts = [], []
    for _ in range(pairs):
        q = rng.integers(0, 4, m, dtype=np.uint8)
        ps.append(q)
        ts.append(simulate(q, 0.10, ONT_INDEL, rng))
    return _assemble(ps, ts, np.full(pairs, band), "c2")


def c3_band(L: np.ndarray) -> np.ndarray:
    """Band for a query of L bases: clamp(32 * ceil(0.1 * L / 32), 64, 512)."""
    return np.clip(32 * np.ceil(0.1 * L / 32.0), 64, 512).astype(np.uint64)


def config3(pairs: int = 100_000, seed: int = 3) -> tuple[Pairs, Pairs]:
    """(Myers pairs with flanked targets, affine pairs) for the same queries."""
    rng = np.random.default_rng(seed)
    L = np.clip(np.round(np.exp(np.log(1200.0) + 0.8 * rng.standard_normal(pairs))), 200,
                20000).astype(np.int64)
    rates = rng.uniform(0.05, 0.12, pairs)
    qs, ts, fts = [], [], []
    for i in range(pairs):
        q = rng.integers(0, 4, int(L[i]), dtype=np.uint8)
        t = simulate(q, float(rates[i]), ONT_INDEL, rng)
        fl = rng.integers(0, 4, 100, dtype=np.uint8)
        qs.append(q)
        ts.append(t)
        fts.append(np.concatenate([fl[:50], t, fl[50:]]))
    return (_assemble(qs, fts, np.zeros(pairs), "c3-myers"),
            _assemble(qs, ts, c3_band(L.astype(np.float64)), "c3-affine"))


# ---- serving stream (config 5) ------------------------------------------------------------

ONT_CDNA = Profile(0.40, 0.25, 0.35, 4.0)  # sim.rs:28-35 `ont`


@dataclass
class Read:
    read: np.ndarray     # the read, in the transcript's orientation
    region: np.ndarray   # the transcript bases it came from
    flanked: np.ndarray  # region with 50 random bases on each side


def serving_read(rng: np.random.Generator, hifi: bool) -> Read:
    """One read of the serving model.  ONT cDNA-like reads (7% error, sim.rs `ont` profile)
    cover the 3' end of a transcript of 300..12,000 bases (log-normal, median 1,500): the
    reference simulator keeps the 3' end and truncates the 5' end
    (crates/spearfish-cli/src/simulate_cmd.rs:4-6).  HiFi-like reads are 1..20 kb at 1%
    error."""
    if hifi:
        L = int(rng.integers(1000, 20001))
        region = rng.integers(0, 4, L, dtype=np.uint8)
        read = simulate(region, 0.01, HIFI, rng)
    else:
        T = int(np.clip(np.exp(np.log(1500.0) + 0.6 * rng.standard_normal()), 300, 12000))
        keep = int(T * rng.uniform(0.5, 1.0))
        region = rng.integers(0, 4, keep, dtype=np.uint8)
        read = simulate(region, 0.07, ONT_CDNA, rng)
    fl = rng.integers(0, 4, 100, dtype=np.uint8)
    return Read(read, region, np.concatenate([fl[:50], region, fl[50:]]))


def serving_jobs(reads: list, B) -> tuple[np.ndarray, np.ndarray]:
    """The jobs a read batch hands the alignment stage, per read: a Myers Infix distance of the
    read against its flanked region (map/src/lib.rs:913-935 `whole_read`), a banded Global
    affine pass with CIGAR over the region (band as in the uneven batch), and X-drop
    extensions of its two 100-base ends into windows of x + 20 + x/10 bases
    (map/src/lib.rs:2100-2114 `extend_dp`, TieBreak/Ends defaults: band 16, X-drop 50,
    end bonus 5), with CIGARs."""
    pool = []
    at = 0
    rows = []

    def put(a):
        nonlocal at
        pool.append(a)
        off = at
        at += a.size
        return off

    for r in reads:
        m = r.read.size
        po = put(r.read)
        rows.append((po, m, put(r.flanked), r.flanked.size, B.JOB_MYERS, 0, 0, 0, 0, 0, 0))
        band = int(c3_band(np.array([float(m)]))[0])
        rows.append((po, m, put(r.region), r.region.size, B.JOB_AFFINE, 2, 1, band, 0, 0, 0))
        x = min(100, m)
        w = x + 20 + x // 10
        # right end: the read's last x bases against the region's last w bases
        tail = r.region[max(0, r.region.size - w):]
        rows.append((po + m - x, x, put(tail), tail.size, B.JOB_EXTEND_WINDOW, 1, 1, 16, w,
                     5, 50))
        # left end: reversed, as the mapper extends leftwards (map/src/lib.rs:3266-3274)
        head_r = np.ascontiguousarray(r.read[:x][::-1])
        head_t = np.ascontiguousarray(r.region[:w][::-1])
        rows.append((put(head_r), x, put(head_t), head_t.size, B.JOB_EXTEND_WINDOW, 1, 1, 16,
                     w, 5, 50))
    jobs = B.new_jobs(len(rows))
    for q, (po, m, to, n, kind, mode, cig, band, win, bonus, xd) in enumerate(rows):
        j = jobs[q]
        j["p_off"], j["m"], j["t_off"], j["n"] = po, m, to, n
        j["kind"], j["mode"], j["want_cigar"] = kind, mode, cig
        if kind != B.JOB_MYERS:
            j["band"] = band
        if kind == B.JOB_EXTEND_WINDOW:
            j["window"], j["end_bonus"], j["xdrop"] = win, bonus, xd
    return (np.concatenate(pool) if pool else np.zeros(1, np.uint8)), jobs


class Transcriptome:
    """Seeded transcripts for the served stream over the transcript store: ONT-like
    transcripts of 300..12,000 bases (log-normal, median 1,500) and, for the HiFi-like 10%,
    longer ones of 1..20 kb.  `starts` are their first bases in the concatenation (as the
    index's `tx_range` numbers them)."""

    def __init__(self, n_ont: int = 20_000, n_long: int = 1_000, seed: int = 55):
        rng = np.random.default_rng(seed)
        lens = np.clip(np.exp(np.log(1500.0) + 0.6 * rng.standard_normal(n_ont)), 300, 12000)
        self.ont = [rng.integers(0, 4, int(L), dtype=np.uint8) for L in lens]
        self.long = [rng.integers(0, 4, int(rng.integers(1000, 20001)), dtype=np.uint8)
                     for _ in range(n_long)]
        self.txs = self.ont + self.long
        sizes = np.array([t.size for t in self.txs], dtype=np.uint64)
        self.starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)


def serving_store_read(tx: Transcriptome, rng: np.random.Generator, hifi: bool):
    """A read of the served stream drawn from a stored transcript: ONT cDNA-like reads cover
    the transcript's 3' end (the reference simulator keeps the 3' end,
    crates/spearfish-cli/src/simulate_cmd.rs:4-6) at 7% error; HiFi-like reads cover a long
    transcript at 1%.  Returns (read codes, transcript index, region start, region end)."""
    if hifi:
        x = len(tx.ont) + int(rng.integers(0, len(tx.long)))
        t = tx.txs[x]
        a, b = 0, t.size
        read = simulate(t, 0.01, HIFI, rng)
    else:
        x = int(rng.integers(0, len(tx.ont)))
        t = tx.txs[x]
        a, b = t.size - int(t.size * rng.uniform(0.5, 1.0)), t.size
        read = simulate(t[a:b], 0.07, ONT_CDNA, rng)
    return read, x, a, b


def serving_store_jobs(tx: Transcriptome, reads: list, B) -> tuple[np.ndarray, np.ndarray]:
    """`serving_jobs` with the texts named as windows of the transcript store: the Myers
    Infix distance against the region with up to 50 transcript bases either side, the banded
    Global pass over the region and the right-end extension read their text from the store;
    only the reads (and the reversed left-end window, which the store holds forwards) go in
    the request's pool."""
    pool, at, rows = [], 0, []

    def put(a):
        nonlocal at
        pool.append(a)
        off = at
        at += a.size
        return off

    S, P = B.TEXT_STORE, B.TEXT_POOL
    for read, x, a, b in reads:
        t = tx.txs[x]
        s0 = int(tx.starts[x])
        m = read.size
        po = put(read)
        fa, fb = max(0, a - 50), min(t.size, b + 50)
        rows.append((po, m, s0 + fa, fb - fa, S, B.JOB_MYERS, 0, 0, 0, 0, 0, 0))
        band = int(c3_band(np.array([float(m)]))[0])
        rows.append((po, m, s0 + a, b - a, S, B.JOB_AFFINE, 2, 1, band, 0, 0, 0))
        xr = min(100, m)
        w = xr + 20 + xr // 10
        ta = max(a, b - w)
        rows.append((po + m - xr, xr, s0 + ta, b - ta, S, B.JOB_EXTEND_WINDOW, 1, 1, 16, w, 5, 50))
        head_r = np.ascontiguousarray(read[:xr][::-1])
        head_t = np.ascontiguousarray(t[a:min(b, a + w)][::-1])
        rows.append((put(head_r), xr, put(head_t), head_t.size, P, B.JOB_EXTEND_WINDOW, 1, 1, 16,
                     w, 5, 50))
    jobs = B.new_jobs(len(rows))
    for q, (po, m, to, n, src, kind, mode, cig, band, win, bonus, xd) in enumerate(rows):
        j = jobs[q]
        j["p_off"], j["m"], j["t_off"], j["n"], j["text_src"] = po, m, to, n, src
        j["kind"], j["mode"], j["want_cigar"] = kind, mode, cig
        if kind != B.JOB_MYERS:
            j["band"] = band
        if kind == B.JOB_EXTEND_WINDOW:
            j["window"], j["end_bonus"], j["xdrop"] = win, bonus, xd
    return (np.concatenate(pool) if pool else np.zeros(1, np.uint8)), jobs


def serving_stream(duration_s: float, reads_per_s: float = 2000.0, burst: float = 5.0,
                   max_batch: int = 4096, seed: int = 5, exact_mean: bool = True):
    """Arrivals of read batches: batch sizes log-uniform over 1..max_batch reads, batch
    arrivals Poisson, the rate switching between a base rate and `burst` times it (bursts of
    exponential length, mean 0.5 s, 10% of the time) so that the mean is `reads_per_s`.
    A window of seconds holds few batches of very uneven size, so its own mean drifts far
    from the stream's; with `exact_mean` the arrival times are scaled so that the window
    offers exactly `reads_per_s` (reads / last arrival).
    Returns [(arrival seconds, reads in the batch)]."""
    rng = np.random.default_rng(seed)
    mean_batch = (max_batch - 1) / np.log(max_batch)
    base = reads_per_s / mean_batch / (0.9 + 0.1 * burst)
    t, out, bursting, switch = 0.0, [], False, rng.exponential(4.5)
    while t < duration_s:
        rate = base * (burst if bursting else 1.0)
        dt = rng.exponential(1.0 / rate)
        if t + dt > switch:
            t = switch
            bursting = not bursting
            switch = t + rng.exponential(0.5 if bursting else 4.5)
            continue
        t += dt
        size = int(np.clip(np.round(np.exp(rng.uniform(0, np.log(max_batch)))), 1, max_batch))
        out.append((t, size))
    if exact_mean and out:
        f = sum(n for _, n in out) / reads_per_s / out[-1][0]
        out = [(a * f, n) for a, n in out]
    return out
