"""Parity of the CUDA library (through the C ABI) with the oracle and the reference's known
answers: bit-exact distances, scores, end cells and CIGARs.

The reference's own tests are replayed against the GPU -- its KATs, the shrunk inputs in its
proptest-regressions file, and its property families (align.rs:3045-3500) on seeded inputs --
once through the one-call entry points (the drop-in boundary) and once through batched plans
(every kernel class: register rows of C = 4..48 cells per lane, wide rows, Myers segments of
1..32 lanes and 1..16 blocks per lane)."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from spearfish_gb300 import build
    build.build()
    return R.GpuImpl()


@pytest.fixture(scope="module")
def ctx(gpu):
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield c
    c.close()


# ---- helpers -------------------------------------------------------------------------

class Jobs:
    """Collects jobs for one batched plan and the oracle's answer for each."""

    def __init__(self):
        from spearfish_gb300 import batch as B
        self.B = B
        self.pool = B.PoolBuilder()
        self.rows = []
        self.want = []

    def add(self, want, **f):
        p, t = f.pop("p"), f.pop("t")
        f["p_off"] = self.pool.add(p)
        f["m"] = len(p)
        f["t_off"] = self.pool.add(t)
        f["n"] = len(t)
        self.rows.append(f)
        self.want.append(want)

    def run(self, ctx, scores=(R.ONT,)):
        jobs = self.B.new_jobs(len(self.rows))
        for q, f in enumerate(self.rows):
            for k, v in f.items():
                jobs[q][k] = v
        return self.B.run(ctx, self.pool.build(), jobs, scores)


def myers_case(rng):
    if rng.random() < 0.5:
        p = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
        t = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
    else:
        p, t = R.related(rng)
    return p, t


# ---- known answers and regressions ------------------------------------------------

def test_kats(gpu):
    R.check_kats(gpu)


def test_extend_kat_equals_naive(gpu):
    for c in R.golden()["kats"]:
        if c["fn"] == "affine_extend_vs_naive":
            a = c["args"]
            assert gpu.affine_extend(a["p"], a["t"], a["sc"], a["band"], a["end_bonus"],
                                     a["xdrop"]) == O.naive_extend(a["p"], a["t"], a["sc"])


def test_window_relations(gpu):
    R.check_window_relations(gpu)


def test_regressions(gpu):
    for c in R.golden()["regressions"]:
        a = c["args"]
        if c["test"] == "random_vs_naive":
            for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
                want = O.myers_naive(a["p"], a["t"], mode)
                assert gpu.distance(a["p"], a["t"], mode, a["k"]) == (want if want <= a["k"]
                                                                      else None)
        elif c["test"] == "related_vs_naive":
            t = a["t"]
            end = min(a["a"] + a["len"], len(t))
            p = R.mutate(t[min(a["a"], end):end], a["edits"])
            d = O.myers_naive(p, t, R.INFIX)
            for k in (max(d - 1, 0), d, d + a["slack"], R.U32_MAX):
                for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
                    want = O.myers_naive(p, t, mode)
                    assert gpu.distance(p, t, mode, k) == (want if want <= k else None)
        elif c["test"] == "local_band_matches_definition":
            b = a["bonus"] if isinstance(a["bonus"], list) else [a["bonus"], a["bonus"]]
            for sc in (R.ONT, R.HIFI):
                m, n = len(a["p"]), len(a["t"])
                assert gpu.local_band_ends(a["p"], a["t"], sc, -m, n, b) == \
                    O.naive_local(a["p"], a["t"], sc, b)
        elif c["test"] == "sorted_batch_matches_single":
            base = a["base"]
            p = R.mutate(base, a["edits"])
            texts = R.sorted_texts(base, a["variants"])
            _check_sorted(gpu, p, texts, a["band"], a["xdrop"], a["bonus"], a["window_extra"])
        elif c["test"] == "narrow_cells_match_wide":
            _check_narrow(gpu, a)


def _check_sorted(gpu, p, texts, band, xdrop, bonus, window_extra):
    """align.rs:3245-3309 `sorted_batch_matches_single`, GPU against the oracle."""
    for sc in (R.ONT, R.HIFI):
        for mode in (R.GLOBAL, R.PREFIX):
            assert gpu.affine_sorted(p, texts, mode, sc, band) == \
                [O.affine(p, t, mode, sc, band) for t in texts]
        for diag in (False, True):
            got = gpu.affine_extend_sorted_cut_bonus(p, texts, sc, band, bonus, xdrop, diag, 0,
                                                     None, True, False)
            want = O.affine_extend_sorted_cut_bonus(p, texts, sc, band, bonus, xdrop, diag, 0,
                                                    None, True, False)
            assert got == want
        w = max((len(t) for t in texts), default=0) + window_extra
        c = min((len(t) for t in texts), default=0) + window_extra // 2
        for args in ((bonus, xdrop, False, w, None, True, False),
                     (bonus, R.I32_MAX, False, w, c, True, False),
                     (bonus, xdrop, False, w, c, True, True),
                     (bonus, xdrop, True, w, c, False, True)):
            got = gpu.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args)
            want = O.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args)
            assert got == want, args
        for t in texts:
            assert gpu.affine_extend_window(p, t, w, sc, band, bonus, xdrop) == \
                O.affine_extend_window(p, t, w, sc, band, bonus, xdrop)


def _check_narrow(gpu, a):
    """align.rs:3440-3500 `narrow_cells_match_wide`'s inputs: every pass the reference runs
    there, GPU against the oracle (the reference compares 16- and 32-bit cells)."""
    p, t = R.rand_pair(a["n"], a["div"], a["seed"])
    texts = R.narrow_texts(t, a["variants"])
    s = a["scale"]
    sc = (2 * s, 4 * s, 4 * s, 2 * s)
    m = len(p)
    w = max(len(x) for x in texts) + a["window_extra"]
    band = a["band"]
    for mode in (R.GLOBAL, R.PREFIX):
        assert gpu.affine_sorted(p, texts, mode, sc, band) == \
            [O.affine(p, x, mode, sc, band) for x in texts]
    for xdrop in (a["xdrop"] * s, R.I32_MAX):
        for cut in (None, a["cut"]):
            for track in (False, True):
                for diag in (False, True):
                    args = (0, xdrop, diag, 0 if diag else w, cut, track, False)
                    assert gpu.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args) == \
                        O.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args), args
    for x in texts:
        assert gpu.affine_extend_window(p, x, w, sc, band, 5, a["xdrop"] * s) == \
            O.affine_extend_window(p, x, w, sc, band, 5, a["xdrop"] * s)
    _ = m


# ---- Myers -------------------------------------------------------------------------

def test_myers_one_call(gpu):
    rng = np.random.default_rng(101)
    for _ in range(40):
        p, t = myers_case(rng)
        for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
            k = R.U32_MAX if rng.random() < 0.4 else int(rng.integers(0, 400))
            assert gpu.distance(p, t, mode, k) == O.myers_distance(p, t, mode, k)


def test_myers_batch_distances(gpu):
    rng = np.random.default_rng(102)
    for _ in range(10):
        base = rng.integers(0, 4, int(rng.integers(1, 700))).tolist()
        p = R.mutate(base[:int(rng.integers(0, 500))], R.rand_edits(rng, 20, 700))
        texts = [R.mutate(base[int(rng.integers(0, 100)):], R.rand_edits(rng, 25, 700))
                 for _ in range(int(rng.integers(1, 20)))]
        for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
            k = R.U32_MAX if rng.random() < 0.5 else int(rng.integers(0, 80))
            assert gpu.batch_distances(p, texts, mode, k) == \
                [O.myers_distance(p, t, mode, k) for t in texts]


def test_myers_every_class(ctx):
    """Patterns of 0..20,000 bases: segments of 1..32 lanes and 1..16 blocks per lane."""
    rng = np.random.default_rng(103)
    J = Jobs()
    lens = [0, 1, 2, 63, 64, 65, 127, 128, 129, 200, 500, 1000, 1024, 1500, 2047, 2048, 2049,
            3000, 4100, 6000, 9000, 12000, 16384, 20000]
    for m in lens:
        for _ in range(3):
            p = rng.integers(0, 4, m).tolist()
            t = R.mutate(p, R.rand_edits(rng, max(1, m // 12), max(1, m)))
            flank = rng.integers(0, 4, int(rng.integers(0, 60))).tolist()
            t = flank + t + flank[::-1]
            if rng.random() < 0.2:
                t = t[:int(rng.integers(0, len(t) + 1))]
            mode = int(rng.integers(0, 3))
            k = R.U32_MAX if rng.random() < 0.6 else int(rng.integers(0, max(2, m // 4)))
            J.add(O.myers_distance(p, t, mode, k), p=p, t=t, kind=0, mode=mode, k=k)
    out = J.run(ctx)
    got = [None if d == R.U32_MAX else int(d) for d in out.results["distance"]]
    assert got == J.want


# ---- affine ------------------------------------------------------------------------

def test_affine_one_call(gpu):
    rng = np.random.default_rng(104)
    for it in range(25):
        p, t = R.affine_case(rng)
        sc = R.ONT if it % 2 else R.HIFI
        for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
            for band in (None, 0, 1, 8, 400):
                assert gpu.affine(p, t, mode, sc, band) == O.affine(p, t, mode, sc, band)
        if len(p) <= 40 and len(t) <= 60:
            assert gpu.affine_extend(p, t, sc, None, 0, R.I32_MAX) == O.naive_extend(p, t, sc)


def test_affine_every_class(ctx):
    """Bands from 0 to 900 (register rows of every C, and wide rows), every mode, extend
    windows with X-drop, against the oracle's `run_core`."""
    rng = np.random.default_rng(105)
    J = Jobs()
    bands = [0, 1, 3, 10, 30, 60, 100, 150, 190, 250, 380, 500, 700, 760, 800, 900, None]
    for band in bands:
        for _ in range(4):
            m = int(rng.integers(0, 1400))
            p, t = R.rand_pair(m, int(rng.integers(4, 30)), int(rng.integers(1, 2 ** 62)))
            if rng.random() < 0.3:
                t = t[:int(rng.integers(0, len(t) + 1))]
            sc = R.ONT if rng.random() < 0.5 else R.HIFI
            sci = 0 if sc == R.ONT else 1
            mode = int(rng.integers(0, 3))
            J.add((O.affine(p, t, mode, sc, band), None),
                  p=p, t=t, kind=1, mode=mode, band=2 ** 64 - 1 if band is None else band,
                  sc_index=sci)
            w = len(t) + int(rng.integers(0, 200))
            xd = int(rng.integers(0, 120)) if rng.random() < 0.8 else R.I32_MAX
            bonus = int(rng.integers(0, 10))
            J.add((None, O.affine_extend_window(p, t, w, sc, band, bonus, xd)),
                  p=p, t=t, kind=2, band=2 ** 64 - 1 if band is None else band, window=w,
                  xdrop=xd, end_bonus=bonus, sc_index=sci)
    out = J.run(ctx, scores=(R.ONT, R.HIFI))
    r = out.results
    for q, (aff, ext) in enumerate(J.want):
        if aff is not None:
            assert int(r["score"][q]) == aff, (q, J.rows[q])
        else:
            got = (int(r["score"][q]), int(r["pattern_end"][q]), int(r["text_end"][q]),
                   int(r["text_read"][q]))
            assert got == ext, (q, J.rows[q]["band"])


def test_affine_infix_wide_rows(ctx):
    """Unbanded Infix passes over texts longer than the register rows (wide kernel)."""
    rng = np.random.default_rng(106)
    J = Jobs()
    for n in (1535, 1536, 1537, 3000, 5200):
        for _ in range(2):
            t = rng.integers(0, 4, n).tolist()
            a = int(rng.integers(0, n // 2))
            p = R.mutate(t[a:a + int(rng.integers(50, 400))], R.rand_edits(rng, 20, 400))
            J.add(O.affine(p, t, R.INFIX, R.ONT, None), p=p, t=t, kind=1, mode=R.INFIX)
    out = J.run(ctx)
    assert [int(s) for s in out.results["score"]] == J.want


def test_extend_and_sorted_one_call(gpu):
    rng = np.random.default_rng(107)
    for _ in range(6):
        base = rng.integers(0, 4, int(rng.integers(1, 160))).tolist()
        p = R.mutate(base, R.rand_edits(rng, int(rng.integers(0, 12)), 160))
        variants = [(int(rng.integers(0, 160)), rng.integers(0, 4, int(rng.integers(0, 40))).tolist(),
                     int(rng.integers(0, 60))) for _ in range(int(rng.integers(1, 8)))]
        texts = R.sorted_texts(base, variants)
        _check_sorted(gpu, p, texts, int(rng.integers(2, 24)), int(rng.integers(5, 60)),
                      int(rng.integers(0, 8)), int(rng.integers(0, 40)))


# ---- local band ----------------------------------------------------------------------

def test_local_band(gpu):
    rng = np.random.default_rng(108)
    for _ in range(60):
        p = rng.integers(0, 4, int(rng.integers(0, 8))).tolist()
        t = rng.integers(0, 4, int(rng.integers(0, 8))).tolist()
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        sc = R.ONT if rng.random() < 0.5 else R.HIFI
        m, n = len(p), len(t)
        assert gpu.local_band_ends(p, t, sc, -m, n, b) == O.naive_local(p, t, sc, b)
    for _ in range(40):
        base = rng.integers(0, 4, int(rng.integers(1, 300))).tolist()
        p = base[int(rng.integers(0, len(base))):]
        p = R.mutate(p, R.rand_edits(rng, int(rng.integers(0, 30)), 300, base_max=5))
        p = rng.integers(0, 4, int(rng.integers(0, 30))).tolist() + p
        dlo, width = int(rng.integers(-320, 320)), int(rng.integers(0, 200))
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        sc = R.ONT if rng.random() < 0.5 else R.HIFI
        assert gpu.local_band_ends(p, base, sc, dlo, dlo + width, b) == \
            O.naive_local_band(p, base, sc, dlo, dlo + width, b)


def test_local_band_plan(ctx):
    rng = np.random.default_rng(109)
    J = Jobs()
    for _ in range(120):
        base = rng.integers(0, 4, int(rng.integers(1, 2500))).tolist()
        p = base[int(rng.integers(0, len(base))):][:int(rng.integers(1, 1500))]
        p = R.mutate(p, R.rand_edits(rng, int(rng.integers(0, 40)), 2000, base_max=5))
        dlo = int(rng.integers(-200, 200))
        width = int(rng.integers(0, 1800))
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        sc = R.ONT if rng.random() < 0.5 else R.HIFI
        J.add(O.local_band_ends(p, base, sc, dlo, dlo + width, b), p=p, t=base, kind=3,
              dlo=dlo, dhi=dlo + width, end_bonus=b[0], end_bonus2=b[1],
              sc_index=0 if sc == R.ONT else 1)
    out = J.run(ctx, scores=(R.ONT, R.HIFI))
    assert [int(s) for s in out.results["score"]] == J.want


# ---- CIGARs --------------------------------------------------------------------------

def test_cigar_one_call(gpu):
    from spearfish_gb300 import align as A
    rng = np.random.default_rng(110)
    for it in range(30):
        p, t = R.rand_pair(int(rng.integers(1, 500)), int(rng.integers(3, 20)),
                           int(rng.integers(1, 2 ** 62)))
        sc = R.ONT if it % 2 else R.HIFI
        band = [None, 8, 16, 64, 200][it % 5]
        for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
            g = A.affine_cigar(p, t, mode, sc, band)
            o = O.traceback(p, t, O.TB_AFFINE, mode, sc, band)
            assert (g["score"], g["status"], g["pattern_end"], g["text_end"]) == \
                (o["score"], o["status"], o["end_i"], o["end_j"])
            if o["status"] == 0:
                assert g["cigar"] == o["cigar"], (mode, band)
                assert g["text_start"] == o["text_start"]
        w = len(t) + int(rng.integers(0, 50))
        xd, bonus = int(rng.integers(5, 80)), int(rng.integers(0, 8))
        g = A.affine_extend_window_cigar(p, t, w, sc, band, bonus, xd)
        o = O.traceback(p, t, O.TB_EXTEND, O.PREFIX, sc, band, w, bonus, xd)
        assert (g["score"], g["status"], g["pattern_end"], g["text_end"], g["cigar"]) == \
            (o["score"], o["status"], o["end_i"], o["end_j"], o["cigar"])
    # Rows of up to 1,536 cells (48 cells per lane) through the one-call path.
    for n in (1100, 1500):
        t = rng.integers(0, 4, n).tolist()
        p = R.mutate(t[100:900], R.rand_edits(rng, 60, 800))
        g = A.affine_cigar(p, t, R.INFIX, R.ONT, None)
        o = O.traceback(p, t, O.TB_AFFINE, R.INFIX, R.ONT, None)
        assert (g["score"], g["cigar"], g["text_start"]) == (o["score"], o["cigar"],
                                                            o["text_start"])


def test_cigar_plan_every_class(ctx):
    """CIGARs from every kernel class equal the traceback oracle's and re-score exactly."""
    rng = np.random.default_rng(111)
    J = Jobs()
    for band in (2, 20, 50, 100, 180, 250, 400, 600, 740, 850, None):
        for _ in range(3):
            m = int(rng.integers(1, 1600))
            p, t = R.rand_pair(m, int(rng.integers(4, 25)), int(rng.integers(1, 2 ** 62)))
            mode = int(rng.integers(0, 3))
            J.add(("a", p, t, mode, band), p=p, t=t, kind=1, mode=mode,
                  band=2 ** 64 - 1 if band is None else band, want_cigar=1)
            w = len(t) + int(rng.integers(0, 100))
            xd, bonus = int(rng.integers(10, 100)), int(rng.integers(0, 8))
            J.add(("e", p, t, w, band, bonus, xd), p=p, t=t, kind=2, window=w, xdrop=xd,
                  end_bonus=bonus, band=2 ** 64 - 1 if band is None else band, want_cigar=1)
    out = J.run(ctx)
    for q, w in enumerate(J.want):
        r = out.results[q]
        if w[0] == "a":
            _, p, t, mode, band = w
            o = O.traceback(p, t, O.TB_AFFINE, mode, R.ONT, band)
        else:
            _, p, t, win, band, bonus, xd = w
            o = O.traceback(p, t, O.TB_EXTEND, O.PREFIX, R.ONT, band, win, bonus, xd)
        assert int(r["status"]) == o["status"]
        assert (int(r["score"]), int(r["pattern_end"]), int(r["text_end"])) == \
            (o["score"], o["end_i"], o["end_j"])
        if o["status"] == 0:
            got = out.cigar(q)
            assert got == o["cigar"], (q, w[0], w[-1])
            s, pu, te = O.cigar_score(p, t, got, int(r["text_start"]), R.ONT)
            assert (pu, te) == (len(p), int(r["text_end"]))


# ---- edges and counters ---------------------------------------------------------------

def test_edges(gpu):
    for p, t in (([], []), ([0], []), ([], [1, 2]), ([3], [3]), ([0, 1], [2, 3])):
        for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
            assert gpu.distance(p, t, mode) == O.myers_distance(p, t, mode)
            for band in (None, 0, 1, 5):
                assert gpu.affine(p, t, mode, R.ONT, band) == O.affine(p, t, mode, R.ONT, band)
        assert gpu.affine_extend_window(p, t, 10, R.ONT, 3, 5, 0) == \
            O.affine_extend_window(p, t, 10, R.ONT, 3, 5, 0)
        assert gpu.local_band_ends(p, t, R.ONT, -2, 2, (1, 2)) == \
            O.local_band_ends(p, t, R.ONT, -2, 2, (1, 2))
    # Window far beyond the text: rows run past it by more than the band (early NEG).
    p, t = R.rand_pair(300, 10, 5)
    assert gpu.affine_extend_window(p, t[:50], 400, R.ONT, 4, 5, R.I32_MAX) == \
        O.affine_extend_window(p, t[:50], 400, R.ONT, 4, 5, R.I32_MAX)


def test_dp_work_counts(gpu):
    from spearfish_gb300 import align as A
    p, t = R.rand_pair(900, 10, 77)
    c0, r0 = A.dp_work()
    A.affine(p, t, R.GLOBAL, R.ONT, 50)
    c1, r1 = A.dp_work()
    d = O.affine_dp(p, t, R.GLOBAL, R.ONT, 50)
    assert (c1 - c0, r1 - r0) == (d["cells"], d["rows"])
