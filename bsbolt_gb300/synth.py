"""Seeded synthetic inputs for the bisulfite seed/extend path.

No public dataset is used: every workload is generated here from
``numpy.random.Generator(PCG64(seed))``.  Shapes follow the workloads the
path is measured on:

* ``ksw_jobs`` -- batched ``ksw_extend2`` jobs: query length U[10,140] in the
  three-letter converted alphabet (A/G/T ~ 30/20/50 %, 1 % N), target = the
  query mutated with 1 % substitutions and 0.1 % indels of length 1-5, plus
  100 nt of flank; 20 % of jobs get an unrelated random target so z-drop and
  the zero-row exit fire; h0 ~ U[19,100]; w = 100; end bonus 5.
* ``bs_genome`` / ``bs_reads`` -- a GC-41 % reference with thinned CpG and
  directional paired-end bisulfite reads (see their docstrings).
"""
from __future__ import annotations

import numpy as np

# bsb_ext_job_t in include/bsbgpu.h
JOB_DTYPE = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                      ("h0", "<i4"), ("w", "<i4"), ("end_bonus", "<i4"), ("flags", "<i4")])

NT4 = np.full(256, 4, np.uint8)
for _i, _c in enumerate("ACGT"):
    NT4[ord(_c)] = _i
    NT4[ord(_c.lower())] = _i


def fill_scmat(a: int = 1, b: int = 4) -> np.ndarray:
    """Scoring matrix of bwa_fill_scmat (bsbolt/External/BWA/bwa.c:169-178): a on the
    diagonal, -b off it, -1 against N."""
    mat = np.full((5, 5), -1, np.int8)
    for i in range(4):
        for j in range(4):
            mat[i, j] = a if i == j else -b
    return mat.reshape(25)


def _draw(rng, n, p):
    """n base codes with probabilities p (resolution 1/1024) via a lookup table."""
    p = np.asarray(p, float)
    counts = np.floor(p / p.sum() * 1024 + 0.5).astype(np.int64)
    counts[np.argmax(counts)] += 1024 - counts.sum()
    lut = np.repeat(np.arange(len(p), dtype=np.uint8), counts)
    return lut[rng.integers(0, 1024, n, dtype=np.uint16)]


def _mutate(rng, seq, job_of, n_jobs, sub, indel, alphabet_p):
    """Apply substitutions and indels to a concatenation of per-job sequences.

    Returns (mutated concatenation, per-job lengths).  Deletions never cross a
    job boundary."""
    n = len(seq)
    r = rng.random(n, dtype=np.float32)
    ins = r < indel / 2
    dele = (r >= indel / 2) & (r < indel)
    subm = (r >= indel) & (r < indel + sub)
    out = seq.copy()
    if subm.any():
        k = int(subm.sum())
        # substitute with a different base drawn from the same alphabet
        new = _draw(rng, k, alphabet_p[:4])
        same = new == out[subm]
        new[same] = (new[same] + 1 + rng.integers(0, 3, int(same.sum()))) % 4
        out[subm] = new
    keep = np.ones(n, np.int64)
    if dele.any():
        starts = np.nonzero(dele)[0]
        lens = rng.integers(1, 6, len(starts))
        # clip at the end of the job the deletion starts in
        job_end = np.searchsorted(job_of, job_of[starts], side="right")
        stops = np.minimum(starts + lens, job_end)
        diff = np.zeros(n + 1, np.int64)
        np.add.at(diff, starts, 1)
        np.add.at(diff, stops, -1)
        keep[np.cumsum(diff)[:n] > 0] = 0
    ins_len = np.zeros(n, np.int64)
    if ins.any():
        ins_len[ins] = rng.integers(1, 6, int(ins.sum()))
    per = ins_len + keep
    total = int(per.sum())
    res = np.empty(total, np.uint8)
    pos = np.cumsum(per) - per             # start of each source position's output
    # inserted bases first, then the kept base
    if ins.any():
        ipos = np.nonzero(ins_len)[0]
        idx = np.repeat(pos[ipos], ins_len[ipos]) + (np.arange(int(ins_len[ipos].sum()))
              - np.repeat(np.cumsum(ins_len[ipos]) - ins_len[ipos], ins_len[ipos]))
        res[idx] = _draw(rng, len(idx), alphabet_p)
    kp = keep.astype(bool)
    res[pos[kp] + ins_len[kp]] = out[kp]
    lens = np.bincount(job_of, weights=per, minlength=n_jobs).astype(np.int64)
    return res, lens


def ksw_jobs(n_jobs: int, seed: int = 20261203 + 1, qmin: int = 10, qmax: int = 140,
             flank: int = 100, sub: float = 0.01, indel: float = 0.001,
             unrelated: float = 0.2, h0_range=(19, 100), w: int = 100, end_bonus: int = 5,
             chunk: int = 1 << 18):
    """Batched ksw_extend2 jobs.  Returns (jobs[JOB_DTYPE], seq uint8 buffer).

    Queries and targets are packed back to back in one byte buffer; job i's
    query is seq[qoff:qoff+qlen] and its target seq[toff:toff+tlen]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.array([0.30, 0.0, 0.20, 0.50, 0.01])
    p = p / p.sum()
    jobs_all, parts, base = [], [], 0
    for c0 in range(0, n_jobs, chunk):
        m = min(chunk, n_jobs - c0)
        qlen = rng.integers(qmin, qmax + 1, m).astype(np.int64)
        qtot = int(qlen.sum())
        q = _draw(rng, qtot, p)
        job_of = np.repeat(np.arange(m), qlen)
        mut, mlen = _mutate(rng, q, job_of, m, sub, indel, p)
        unrel = rng.random(m) < unrelated
        # target = mutated query + flank; unrelated jobs get random bases instead
        tlen = mlen + flank
        tlen[unrel] = qlen[unrel] + flank
        t = np.empty(int(tlen.sum()), np.uint8)
        toff_local = np.cumsum(tlen) - tlen
        moff = np.cumsum(mlen) - mlen
        rel = np.nonzero(~unrel)[0]
        body = np.zeros(len(t), bool)
        if len(rel):
            # gather the mutated bodies of related jobs to the front of their targets
            lens_r = mlen[rel]
            within = np.arange(int(lens_r.sum())) - np.repeat(np.cumsum(lens_r) - lens_r, lens_r)
            dst = np.repeat(toff_local[rel], lens_r) + within
            t[dst] = mut[np.repeat(moff[rel], lens_r) + within]
            body[dst] = True
        # everything not yet written (flanks and unrelated bodies) is random
        nfill = int((~body).sum())
        t[~body] = _draw(rng, nfill, p)
        qoff_local = np.cumsum(qlen) - qlen
        js = np.zeros(m, JOB_DTYPE)
        js["qoff"] = base + qoff_local
        js["toff"] = base + qtot + toff_local
        js["qlen"] = qlen
        js["tlen"] = tlen
        js["h0"] = rng.integers(h0_range[0], h0_range[1] + 1, m)
        js["w"] = w
        js["end_bonus"] = end_bonus
        jobs_all.append(js)
        parts.append(q)
        parts.append(t)
        base += qtot + len(t)
    return np.concatenate(jobs_all), np.concatenate(parts)


def cells_upper_bound(jobs: np.ndarray) -> np.ndarray:
    """The plain schedule's cost bound: rows x band columns, qlen x min(tlen, qlen+w)."""
    q = jobs["qlen"].astype(np.int64)
    t = jobs["tlen"].astype(np.int64)
    w = jobs["w"].astype(np.int64)
    return q * np.minimum(t, q + w)


# ---------------------------------------------------------------- genomes / reads

COMP = np.array([3, 2, 1, 0, 4], np.uint8)


def bs_genome(n_contigs: int = 4, contig_len: int = 500_000, gc: float = 0.41,
              cpg_frac: float = 0.01, seed: int = 20261203):
    """i.i.d. contigs at the given GC with CpG thinned to ``cpg_frac`` of dinucleotides.

    Returns a list of (name, codes uint8 0..3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    at = (1 - gc) / 2
    p = np.array([at, gc / 2, gc / 2, at])
    contigs = []
    expect = (gc / 2) ** 2
    keep = min(1.0, cpg_frac / expect)
    for k in range(n_contigs):
        s = _draw(rng, contig_len, p)
        cg = np.nonzero((s[:-1] == 1) & (s[1:] == 2))[0]
        drop = cg[rng.random(len(cg)) >= keep]
        s[drop] = 3                              # thinned CpG: C -> T
        contigs.append((f"chr{k + 1}", s))
    return contigs


def add_repeats(contigs, frac: float = 0.15, fam_len=(300, 6000), div=(0.02, 0.15), n_families: int = 200,
                seed: int = 20261203):
    """Interspersed repeats: copies of `n_families` random families (lengths uniform in
    fam_len), each copy with its own substitution rate uniform in `div`, written over
    random positions until about `frac` of every contig is repeat.  In place; returns
    contigs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    fams = [rng.integers(0, 4, int(rng.integers(fam_len[0], fam_len[1] + 1))).astype(np.uint8)
            for _ in range(n_families)]
    for _, g in contigs:
        covered, target = 0, int(frac * len(g))
        while covered < target:
            f = fams[int(rng.integers(0, n_families))]
            if len(f) >= len(g):
                break
            cp = f.copy()
            if rng.random() < 0.5:
                cp = COMP[cp[::-1]]
            mut = rng.random(len(cp)) < rng.uniform(div[0], div[1])
            cp[mut] = (cp[mut] + rng.integers(1, 4, int(mut.sum()))) % 4
            at = int(rng.integers(0, len(g) - len(cp)))
            g[at:at + len(cp)] = cp
            covered += len(cp)
    return contigs


def write_fasta(path: str, contigs, width: int = 60) -> None:
    letters = np.frombuffer(b"ACGTN", np.uint8)
    with open(path, "wb") as f:
        for name, codes in contigs:
            f.write(f">{name}\n".encode())
            txt = letters[np.asarray(codes, np.uint8)]
            full = len(txt) // width * width
            lines = np.empty((full // width, width + 1), np.uint8)     # whole lines, newline last
            lines[:, :width] = txt[:full].reshape(-1, width)
            lines[:, width] = ord("\n")
            f.write(lines.tobytes())
            if full < len(txt):
                f.write(txt[full:].tobytes() + b"\n")


def bs_reads_pe(contigs, n_pairs: int, read_len: int = 100, insert_mean: float = 300,
                insert_sd: float = 30, meth_cpg: float = 0.8, meth_ch: float = 0.01,
                conversion: float = 0.995, err: float = 0.005, seed: int = 20261203):
    """Directional paired-end bisulfite reads, drawn uniformly from both strands.

    Returns (r1, r2): lists of uint8 code arrays (A0 C1 G2 T3), original bases
    as sequenced, before the aligner's in-silico conversion."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lens = np.array([len(c[1]) for c in contigs], np.float64)
    which = rng.choice(len(contigs), size=n_pairs, p=lens / lens.sum())
    ins = np.maximum(np.round(rng.normal(insert_mean, insert_sd, n_pairs)).astype(np.int64), read_len)
    strand = rng.random(n_pairs) < 0.5           # True: original bottom strand
    r1s, r2s = [], []
    for i in range(n_pairs):
        g = contigs[which[i]][1]
        L = int(min(ins[i], len(g)))
        st = int(rng.integers(0, len(g) - L + 1))
        frag = g[st:st + L].copy()
        if strand[i]:
            frag = COMP[frag[::-1]]
        # methylation and bisulfite conversion on the sequenced strand
        isc = frag == 1
        nxt = np.concatenate([frag[1:], [4]])
        cpg = isc & (nxt == 2)
        meth = np.where(cpg, rng.random(L) < meth_cpg, rng.random(L) < meth_ch)
        conv = isc & ~meth & (rng.random(L) < conversion)
        frag[conv] = 3
        r1 = frag[:read_len].copy()
        r2 = COMP[frag[::-1][:read_len]].copy()
        for r in (r1, r2):
            e = rng.random(len(r)) < err
            r[e] = (r[e] + rng.integers(1, 4, int(e.sum()))) % 4
        r1s.append(r1)
        r2s.append(r2)
    return r1s, r2s


def bs_reads_pe_block(contigs, n_pairs: int, read_len: int = 150, insert_mean: float = 400,
                      insert_sd: float = 50, meth_cpg: float = 0.8, meth_ch: float = 0.01,
                      conversion: float = 0.995, err: float = 0.005, seed: int = 20261203,
                      chunk: int = 250_000):
    """bs_reads_pe's model, vectorised for millions of pairs: directional pairs of read_len
    bases from either strand, insert ~ N(insert_mean, insert_sd) (at least read_len),
    methylation and conversion on the sequenced strand, substitution errors.  Where the two
    reads of a short insert overlap, each draws its own methylation there.  Returns (r1, r2)
    as (n_pairs, read_len) uint8 arrays of bases as sequenced."""
    rng = np.random.Generator(np.random.PCG64(seed))
    G = np.concatenate([np.asarray(c[1], np.uint8) for c in contigs] + [np.full(1, 4, np.uint8)])
    starts = np.cumsum([0] + [len(c[1]) for c in contigs])
    lens = np.diff(starts).astype(np.float64)
    rl = int(read_len)
    j = np.arange(rl, dtype=np.int64)[None, :]
    out1 = np.empty((n_pairs, rl), np.uint8)
    out2 = np.empty((n_pairs, rl), np.uint8)

    def convert(b, nxt):
        u = rng.random(b.shape, dtype=np.float32)
        meth = np.where((b == 1) & (nxt == 2), u < meth_cpg, u < meth_ch)
        conv = (b == 1) & ~meth & (rng.random(b.shape, dtype=np.float32) < conversion)
        b = b.copy()
        b[conv] = 3
        return b

    for lo in range(0, n_pairs, chunk):
        m = min(chunk, n_pairs - lo)
        which = rng.choice(len(contigs), size=m, p=lens / lens.sum())
        ins = np.maximum(np.round(rng.normal(insert_mean, insert_sd, m)).astype(np.int64), rl)
        L = np.minimum(ins, lens[which].astype(np.int64))[:, None]
        s = (starts[which] + (rng.random(m) * (lens[which] - L[:, 0] + 1)).astype(np.int64))[:, None]
        bottom = (rng.random(m) < 0.5)[:, None]
        # the sequenced strand S (top: the contig; bottom: its reverse complement) as positions
        # of G: S[i] = G[s+i] or COMP[G[s+L-1-i]]; read 1 = S[0:rl], read 2 = revcomp(S[L-rl:L])
        def strand(i):
            pos = np.where(bottom, s + L - 1 - i, s + i)
            inside = i < L
            b = G[np.where(inside, pos, len(G) - 1)]
            return np.where(inside & bottom, COMP[b], b)
        a1 = convert(strand(j), strand(j + 1))
        a2 = convert(strand(L - rl + j), strand(L - rl + j + 1))
        r2 = COMP[a2[:, ::-1]]
        for r in (a1, r2):
            e = rng.random(r.shape, dtype=np.float32) < err
            r[e] = (r[e] + rng.integers(1, 4, int(e.sum()), dtype=np.uint8)) % 4
        out1[lo:lo + m], out2[lo:lo + m] = a1, r2
    return out1, out2


def write_fastq_block(path: str, reads, tag: int, first: int = 0, qual: int = ord("?")) -> None:
    """FASTQ of equal-length reads ((n, L) codes 0..4), names @r<9-digit index>/<tag>,
    every quality `qual` (Phred 30 by default), written with fixed-width records."""
    reads = np.asarray(reads, np.uint8)
    n, L = reads.shape
    letters = np.frombuffer(b"ACGTN", np.uint8)
    rec = 18 + 2 * L
    with open(path, "wb") as f:
        for lo in range(0, n, 200_000):
            m = min(200_000, n - lo)
            buf = np.empty((m, rec), np.uint8)
            buf[:, 0], buf[:, 1] = ord("@"), ord("r")
            idx = np.arange(first + lo, first + lo + m, dtype=np.int64)
            for d in range(9):
                buf[:, 10 - d] = ord("0") + (idx // 10 ** d) % 10
            buf[:, 11], buf[:, 12], buf[:, 13] = ord("/"), ord("0") + tag, ord("\n")
            buf[:, 14:14 + L] = letters[reads[lo:lo + m]]
            buf[:, 14 + L], buf[:, 15 + L], buf[:, 16 + L] = ord("\n"), ord("+"), ord("\n")
            buf[:, 17 + L:17 + 2 * L] = qual
            buf[:, 17 + 2 * L] = ord("\n")
            f.write(buf.tobytes())


def write_fastq_ragged(path: str, seqs, offs, tag: int = 1, qual: int = ord("?")) -> None:
    """FASTQ of reads of any length (seqs[offs[i]:offs[i+1]], codes 0..4), names as above."""
    letters = np.frombuffer(b"ACGTN", np.uint8)
    txt = letters[np.asarray(seqs, np.uint8)].tobytes()
    with open(path, "wb") as f:
        parts = []
        for i in range(len(offs) - 1):
            a, b = int(offs[i]), int(offs[i + 1])
            parts.append(b"@r%09d/%d\n%s\n+\n%s\n" % (i, tag, txt[a:b], bytes([qual]) * (b - a)))
            if len(parts) >= 100_000:
                f.write(b"".join(parts))
                parts = []
        f.write(b"".join(parts))


def bs_convert(read: np.ndarray, g2a: bool) -> np.ndarray:
    """In-silico conversion of bsConversion (bs_helpers.cpp:18-31): C->T for read 1,
    G->A for read 2."""
    r = read.copy()
    if g2a:
        r[r == 2] = 0
    else:
        r[r == 1] = 3
    return r


def matesw_jobs(n_jobs: int, seed: int = 20261203 + 5, a: int = 1, min_seed_len: int = 19):
    """Jobs shaped like mem_matesw's ksw_align2 calls (bwamem_pair.c:135-151): a mate read of
    30-250 bases (1 % N) against a reference window of the read length plus 20-700 bases,
    which in 4 of 5 jobs holds a copy of the read with 0-15 % substitutions and up to two
    1-5-base indels; the flags mem_matesw passes (KSW_XSUBO | KSW_XSTART | min_seed_len*a,
    plus KSW_XBYTE when qlen*a < 250).  Returns (jobs with qoff, toff, qlen, tlen, xtra,
    pad as int64, int64, int32 x 4; seq)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dt = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"), ("xtra", "<i4"),
                   ("pad", "<i4")])
    jobs = np.zeros(n_jobs, dt)
    parts, off = [], 0
    for k in range(n_jobs):
        L = int(rng.integers(30, 251))
        q = rng.integers(0, 4, L).astype(np.uint8)
        q[rng.random(L) < 0.01] = 4
        wl = int(rng.integers(L + 20, L + 700))
        t = rng.integers(0, 4, wl).astype(np.uint8)
        if k % 5:
            m = q.copy()
            sub = rng.random(L) < float(rng.choice([0.0, 0.01, 0.05, 0.15]))
            m[sub] = rng.integers(0, 4, int(sub.sum()))
            for _ in range(int(rng.choice([0, 0, 1, 2]))):
                at = int(rng.integers(1, len(m) - 1))
                ln = int(rng.integers(1, 6))
                m = (np.concatenate([m[:at], rng.integers(0, 4, ln).astype(np.uint8), m[at:]]) if rng.random() < .5
                     else np.concatenate([m[:at], m[at + ln:]]))
            m = m[:wl]
            at = int(rng.integers(0, wl - len(m) + 1))
            t[at:at + len(m)] = m
        xtra = 0x40000 | 0x80000 | (0x10000 if L * a < 250 else 0) | (min_seed_len * a)
        jobs[k] = (off, off + L, L, wl, xtra, 0)
        parts += [q, t]
        off += L + wl
    return jobs, np.concatenate(parts)


def rrbs_fragments(contigs, frag_len=(40, 220)):
    """MspI fragments (C^CGG cuts) of frag_len[0]..frag_len[1] bases: (contig index, start, end)."""
    out = []
    for k, (_, g) in enumerate(contigs):
        g = np.asarray(g)
        hit = np.nonzero((g[:-3] == 1) & (g[1:-2] == 1) & (g[2:-1] == 2) & (g[3:] == 2))[0] + 1   # cut after the first C
        if len(hit) < 2:
            continue
        ln = np.diff(hit)
        keep = (ln >= frag_len[0]) & (ln <= frag_len[1])
        out += [(k, int(a), int(b)) for a, b in zip(hit[:-1][keep], hit[1:][keep])]
    return out


def rrbs_reads_se(contigs, n_reads: int, read_lens=(75, 100), frag_len=(40, 220), meth_cpg: float = 0.7,
                  meth_ch: float = 0.01, conversion: float = 0.995, err: float = 0.005, seed: int = 20261203,
                  chunk: int = 200_000):
    """RRBS-like directional single-end reads: every read starts at an end of an MspI fragment
    (the top strand's first base or the bottom strand's), is as long as one of read_lens or the
    fragment if shorter, and many reads share a start (fragments are few).  Methylation,
    conversion and errors as in bs_reads_pe.  Returns (bases as sequenced, concatenated; offsets)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    frags = rrbs_fragments(contigs, frag_len)
    if not frags:
        raise ValueError("no MspI fragments in the length range")
    W = max(read_lens)
    # templates: per fragment and strand, the first W bases of the strand's sequence (padded with 4)
    tmpl = np.full((2 * len(frags), W), 4, np.uint8)
    tlen = np.zeros(2 * len(frags), np.int64)
    for i, (k, a, b) in enumerate(frags):
        f = np.asarray(contigs[k][1][a:b], np.uint8)
        for s, seq in enumerate((f, COMP[f[::-1]])):
            n = min(W, len(seq))
            tmpl[2 * i + s, :n] = seq[:n]
            tlen[2 * i + s] = n
    nxt = np.concatenate([tmpl[:, 1:], np.full((len(tmpl), 1), 4, np.uint8)], axis=1)
    is_c, is_cpg = tmpl == 1, (tmpl == 1) & (nxt == 2)
    parts, lens = [], []
    for lo in range(0, n_reads, chunk):
        m = min(chunk, n_reads - lo)
        tid = rng.integers(0, len(tmpl), m)
        L = np.minimum(rng.choice(np.asarray(read_lens), m), tlen[tid])
        r = tmpl[tid].copy()
        u = rng.random((m, W), dtype=np.float32)
        meth = np.where(is_cpg[tid], u < meth_cpg, u < meth_ch)
        conv = is_c[tid] & ~meth & (rng.random((m, W), dtype=np.float32) < conversion)
        r[conv] = 3
        e = (rng.random((m, W), dtype=np.float32) < err) & (r < 4)
        r[e] = (r[e] + rng.integers(1, 4, int(e.sum()), dtype=np.uint8)) % 4
        keep = np.arange(W)[None, :] < L[:, None]
        parts.append(r[keep])
        lens.append(L)
    lens = np.concatenate(lens)
    offs = np.zeros(n_reads + 1, np.int64)
    offs[1:] = np.cumsum(lens)
    return np.concatenate(parts), offs
