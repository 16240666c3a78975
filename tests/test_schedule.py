"""Host-side models of the pair kernels' work splits (no GPU).

The kernel (mf_allpairs.cuh) walks a flat (target block, source tile) step
space split evenly over a grid of CTAs; target blocks cut by a CTA boundary
are finished from FP64 partials by the last CTA to arrive.  This model replays
that control flow for many shapes and checks that every (target block, tile)
pair is computed exactly once, that every partial the reducer reads was
written by the CTA it expects, in the slot it expects, and that the ticket
count equals the number of writers.  A second model covers the pair-symmetric
launch (mf_sympair.cu): its step-to-block-pair map, that every block-sum slot
is written once, and that the finish's row sums equal the direct sums.  A
third covers the FMM's near field once per box pair (mf_fmm.cu): the half
stencil's plane indices, one writer per (plane, box), the read-back taking
exactly what was written, and every unordered box pair covered once.
"""
import itertools
import random


def start(T, G, b):
    return (T * b) // G


def owner(T, G, x):
    return ((x + 1) * G - 1) // T


def simulate(scenes, tile, tbt, G):
    # scenes: list of (nt, ns)
    desc = []
    step = 0
    tbo = 0
    for nt, ns in scenes:
        n_tiles = -(-ns // tile)
        n_tb = -(-nt // tbt)
        desc.append(dict(nt=nt, ns=ns, n_tiles=n_tiles, n_tb=n_tb, step_off=step, tb_off=tbo))
        step += n_tiles * n_tb
        tbo += n_tb
    T = step
    G = min(G, T)
    computed = {}
    partials = {}  # (block, slot) -> gtb
    tickets = {}
    finished = {}
    for b in range(G):
        kb, ke = start(T, G, b), start(T, G, b + 1)
        assert kb < ke
        # find scene
        si = max(i for i, d in enumerate(desc) if d["step_off"] <= kb)
        local = kb - desc[si]["step_off"]
        tb = local // desc[si]["n_tiles"]
        t = local % desc[si]["n_tiles"]
        seg_from_start = t == 0
        first_tb = True
        for k in range(kb, ke):
            d = desc[si]
            key = (si, tb, t)
            assert key not in computed
            computed[key] = b
            last_tile = t == d["n_tiles"] - 1
            last_step = k == ke - 1
            if last_tile or last_step:
                gtb = d["tb_off"] + tb
                if seg_from_start and last_tile:
                    assert gtb not in finished
                    finished[gtb] = "direct"
                else:
                    slot = 0 if first_tb else 1
                    assert (b, slot) not in partials
                    partials[(b, slot)] = gtb
                    sa = d["step_off"] + tb * d["n_tiles"]
                    se = sa + d["n_tiles"]
                    bf, bl = owner(T, G, sa), owner(T, G, se - 1)
                    nseg = bl - bf + 1
                    tickets[gtb] = tickets.get(gtb, 0) + 1
                    if tickets[gtb] == nseg:
                        first_split = start(T, G, bf) < sa
                        for bb in range(bf, bl + 1):
                            sl = 1 if (bb == bf and first_split) else 0
                            assert partials.get((bb, sl)) == gtb, (bb, sl, gtb)
                        assert gtb not in finished
                        finished[gtb] = "reduced"
                if not last_step:
                    first_tb = False
                    seg_from_start = True
                    t = 0
                    tb += 1
                    if tb == d["n_tb"]:
                        tb = 0
                        si += 1
            else:
                t += 1
    total = sum(d["n_tiles"] * d["n_tb"] for d in desc)
    assert len(computed) == total
    assert len(finished) == tbo, (len(finished), tbo)


def test_single_scene_shapes():
    for n in (1, 2, 3, 31, 33, 255, 256, 257, 511, 512, 513, 4096, 65536):
        for G in (1, 2, 7, 152, 304, 1216):
            simulate([(n, n)], 256, 512, G)


def test_target_source_mismatch():
    for nt, ns in itertools.product((1, 5, 600, 5000), (1, 3, 300, 7000)):
        for G in (3, 152, 304):
            simulate([(nt, ns)], 256, 256, G)


def test_many_scenes():
    rng = random.Random(7)
    for trial in range(20):
        scenes = [(n, n) for n in (int(rng.uniform(1, 5000)) for _ in range(rng.randint(1, 40)))]
        for G in (1, 13, 152, 304, 608):
            simulate(scenes, 256, 512, G)


# ---------------------------------------------------------------------------
# The pair-symmetric launch (mf_sympair.cu): steps are the block pairs
# (I, J), I <= J, row by row; step I < J writes the target-side block sums
# into part[I][J] and the (negated, for the force) source-side ones into
# part[J][I]; a diagonal step writes part[I][I] from every ordered pair.  The
# finish adds, per particle, the nb entries of its block's row.
# ---------------------------------------------------------------------------
import math

import numpy as np


def sym_block_pair(l, nb):
    """Step l -> (I, J), as the device computes it (double sqrt, then exact
    integer corrections)."""
    b = 2.0 * nb + 1.0
    i = int((b - math.sqrt(b * b - 8.0 * l)) * 0.5)
    i = min(max(i, 0), nb - 1)

    def row_start(r):
        return r * nb - r * (r - 1) // 2

    while i > 0 and row_start(i) > l:
        i -= 1
    while i < nb - 1 and row_start(i + 1) <= l:
        i += 1
    return i, i + (l - row_start(i))


def test_sym_block_pairs_are_a_bijection():
    for nb in list(range(1, 130)) + [511]:
        steps = nb * (nb + 1) // 2
        seen = [sym_block_pair(l, nb) for l in range(steps)]
        want = [(i, j) for i in range(nb) for j in range(i, nb)]
        assert seen == want, nb
    # large scenes: the first and last step of every row
    for nb in (1024, 4097, 65536):
        l = 0
        for i in range(nb):
            assert sym_block_pair(l, nb) == (i, i)
            l += nb - i
            assert sym_block_pair(l - 1, nb) == (i, nb - 1)


def sym_plan(sizes, tb):
    out, step, blocks, off = [], 0, 0, 0
    for n in sizes:
        nb = -(-n // tb)
        out.append(dict(n=n, off=off, nb=nb, step_off=step, tb_off=blocks))
        step += nb * (nb + 1) // 2
        blocks += nb * nb
        off += n + (n & 1)  # scenes start at even indices
    return out, step, blocks


def test_sym_partial_slots_written_once():
    rng = random.Random(5)
    for trial in range(40):
        tb = rng.choice([64, 512, 1024])
        sizes = [rng.randint(1, 5 * tb) for _ in range(rng.randint(1, 6))]
        plan, T, blocks = sym_plan(sizes, tb)
        G = rng.randint(1, 700)
        G = min(G, T)
        writes = [0] * blocks
        done = [0] * T
        for b in range(G):
            for k in range(start(T, G, b), start(T, G, b + 1)):
                done[k] += 1
                sc = max((s for s in plan if s["step_off"] <= k), key=lambda s: s["step_off"])
                I, J = sym_block_pair(k - sc["step_off"], sc["nb"])
                writes[sc["tb_off"] + I * sc["nb"] + J] += 1
                if I != J:
                    writes[sc["tb_off"] + J * sc["nb"] + I] += 1
        assert all(d == 1 for d in done)
        assert all(w == 1 for w in writes)


def test_sym_sums_equal_the_direct_sums():
    # Antisymmetric pair values (the force) with the source side negated,
    # and symmetric ones (the field) taken as they are: the finish's row sum
    # per particle equals the direct sum over all partners.
    rng = np.random.default_rng(3)
    tb = 8
    for sizes in ([1], [7], [8], [17, 2, 31], [40]):
        plan, T, blocks = sym_plan(sizes, tb)
        for sign in (-1.0, 1.0):
            for sc in plan:
                n, nb = sc["n"], sc["nb"]
                a, c = rng.normal(size=n), rng.normal(size=n)
                f = np.outer(a, c) + sign * np.outer(c, a)  # f[i, j] = sign * f[j, i]
                if sign < 0:
                    np.fill_diagonal(f, 0.0)
                part = np.full((nb, nb, tb), np.nan)
                for l in range(nb * (nb + 1) // 2):
                    I, J = sym_block_pair(l, nb)
                    ti = np.arange(I * tb, min((I + 1) * tb, n))
                    sj = np.arange(J * tb, min((J + 1) * tb, n))
                    part[I, J, : len(ti)] = f[np.ix_(ti, sj)].sum(axis=1)  # target side
                    if I != J:
                        # source side: sum over the targets of f[i, j], times the
                        # body's source sign (f[j, i] = sign * f[i, j])
                        part[J, I, : len(sj)] = sign * f[np.ix_(ti, sj)].sum(axis=0)
                for i in range(n):
                    K, r = divmod(i, tb)
                    got = part[K, :, r].sum()
                    assert abs(got - f[i].sum()) < 1e-9 * (1 + np.abs(f[i]).sum())


# ---------------------------------------------------------------------------
# The FMM's near field of the force once per unordered box pair (mf_fmm.cu):
# half-stencil rows from the near rows, plane indices, writers and readers.
# ---------------------------------------------------------------------------
def near_rows(R, radius):
    """Rows (w, dy, dz) of a symmetric near stencil: |d| <= radius (box units)."""
    rows = []
    for dz in range(-R, R + 1):
        for dy in range(-R, R + 1):
            if dy * dy + dz * dz > radius * radius:
                continue
            w = 0
            while w + 1 <= R and (w + 1) ** 2 + dy * dy + dz * dz <= radius * radius:
                w += 1
            rows.append((w, dy, dz))
    return rows


def half_rows(rows):
    """As Fmm::build lays them out: (w, dy, dz, planes before the row)."""
    out, n_off = [], 0
    for w, dy, dz in rows:
        if dz > 0 or (dz == 0 and dy > 0):
            out.append((w, dy, dz, n_off))
            n_off += 2 * w + 1
        elif dy == 0 and dz == 0 and w > 0:
            out.append((w, 0, 0, n_off))
            n_off += w
    return out, n_off


def near_plane(hr, dx):
    w, dy, dz, base = hr
    return 1 + base + ((dx - 1) if (dy == 0 and dz == 0) else (dx + w))


def test_fmm_half_stencil_planes():
    rng = random.Random(17)
    for trial in range(30):
        R = rng.randint(1, 4)
        radius = rng.uniform(0.9, R + 0.5)
        rows = near_rows(R, radius)
        hrows, n_off = half_rows(rows)
        nx, ny, nz = rng.randint(1, 7), rng.randint(1, 7), rng.randint(1, 7)
        occupied = {(x, y, z) for x in range(nx) for y in range(ny) for z in range(nz) if rng.random() < 0.7}
        inside = lambda x, y, z: 0 <= x < nx and 0 <= y < ny and 0 <= z < nz  # noqa: E731
        writes, pairs = {}, set()
        for (ax, ay, az) in occupied:  # writer boxes (k_fmm_near_sym)
            for hr in hrows:
                w, dy, dz, _ = hr
                for dx in range(1 if (dy == 0 and dz == 0) else -w, w + 1):
                    b = (ax + dx, ay + dy, az + dz)
                    if not inside(*b) or b not in occupied:
                        continue
                    o = near_plane(hr, dx)
                    assert 1 <= o <= n_off
                    assert (o, b) not in writes
                    writes[(o, b)] = (ax, ay, az)
                    pairs.add(frozenset([(ax, ay, az), b]))
        reads = set()
        for (bx, by, bz) in occupied:  # the read-back in k_fmm_p2p<Q, 1, true>
            for hr in hrows:
                w, dy, dz, _ = hr
                for dx in range(1 if (dy == 0 and dz == 0) else -w, w + 1):
                    a = (bx - dx, by - dy, bz - dz)
                    if inside(*a) and a in occupied:
                        reads.add((near_plane(hr, dx), (bx, by, bz)))
        assert reads == set(writes)
        # every unordered pair of distinct boxes in the full stencil, once
        full = set()
        for (ax, ay, az) in occupied:
            for w, dy, dz in rows:
                for dx in range(-w, w + 1):
                    b = (ax + dx, ay + dy, az + dz)
                    if b != (ax, ay, az) and inside(*b) and b in occupied:
                        full.add(frozenset([(ax, ay, az), b]))
        assert pairs == full


# ---------------------------------------------------------------------------
# The warp reduce-scatter of the source sums (mf_sym.cuh warp_reduce_scatter)
# and the per-warp phase buffer of the fused field-and-force launch
# (mf_sympair.cu k_sym_ff): which lane ends with which sum, and which slot
# each value is stored at and read back from.
# ---------------------------------------------------------------------------
def warp_reduce_scatter(v):
    """Lane-by-lane model of the device's shuffle tree over v[32][NV]."""
    w = np.array(v, dtype=np.float64)
    nv = w.shape[1]
    b, n = 16, nv
    while n > 1:
        new = w.copy()
        for lane in range(32):
            hi = bool(lane & b)
            p = lane ^ b
            phi = bool(p & b)
            for q in range(n // 2):
                keep = w[lane, q + n // 2] if hi else w[lane, q]
                got = w[p, q] if phi else w[p, q + n // 2]  # the partner's `send`
                new[lane, q] = keep + got
        w = new
        n //= 2
        b >>= 1
    while b >= 1:
        w[:, 0] = w[:, 0] + w[np.arange(32) ^ b, 0]
        b >>= 1
    return w[:, 0]


def test_warp_reduce_scatter_lanes():
    rng = np.random.default_rng(9)
    for nv in (8, 16, 32):
        v = rng.normal(size=(32, nv))
        got = warp_reduce_scatter(v)
        per = 32 // nv
        for lane in range(32):
            assert abs(got[lane] - v[:, lane // per].sum()) < 1e-12, (nv, lane)


def test_fused_phase_buffer_slots():
    # k_sym_ff: per pair item 12 values (field x, y, z then force x, y, z, each
    # for the item's two sources: value 2c + s and 6 + 2c + s) in a 16-value
    # reduce-scatter, so value k sits in lanes 2k and 2k + 1 and the even lane
    # stores it at row stride 13.  At the phase's end thread r reads source
    # 2 (r >> 1) + (r & 1) of the phase.  Every (item, value) slot is written
    # once and read once, by the thread of its own source and component.
    TB, SPLIT, ROW = 1024, 4, 13
    NH = TB // 2 // SPLIT
    written, read = {}, {}
    for j in range(NH):
        for lane in range(32):
            kv = lane >> 1
            if lane & 1 == 0 and kv < 12:
                slot = j * ROW + kv
                assert slot not in written
                written[slot] = (j, kv)
    assert len(written) == 12 * NH and max(written) < NH * ROW
    for r in range(2 * NH):
        j, s = r >> 1, r & 1
        for c in range(3):
            for base, prod in ((0, "field"), (6, "force")):
                slot = j * ROW + base + 2 * c + s
                assert slot not in read
                read[slot] = (prod, 2 * j + s, c)
                # the value stored there is that source's component of that product
                assert written[slot] == (j, base + 2 * c + s)
    assert set(read) == set(written)
