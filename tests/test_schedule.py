"""Host-side model of the all-pairs kernel's work split (no GPU).

The kernel (mf_allpairs.cuh) walks a flat (target block, source tile) step
space split evenly over a grid of CTAs; target blocks cut by a CTA boundary
are finished from FP64 partials by the last CTA to arrive.  This model replays
that control flow for many shapes and checks that every (target block, tile)
pair is computed exactly once, that every partial the reducer reads was
written by the CTA it expects, in the slot it expects, and that the ticket
count equals the number of writers.
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
