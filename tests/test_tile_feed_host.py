"""The persistent kernels' tile order (lbmminiapp_gb300/csrc/lbm_launch.cuh),
modelled on the CPU: warps interleaved at random between their counter
atomics, in the three loop shapes the kernels use (compact even step: two
tiles held; compact odd step: four; dense and adjacency-list kernels: three).
Every tile is processed exactly once, whatever the interleaving, the group
count or the chunk size, and the counters are zero again after the launch."""
import random

import pytest

FEED_MIN_TILES = 16


def launch(ntiles, nw, shape, groups, chunk, warps_per_block, seed):
    rng = random.Random(seed)
    ng = min(groups, nw)
    nblocks = nw // warps_per_block
    counters = [0] * (ng + 1)   # group counters, then the finished-block count
    done_warps = [0] * nblocks
    got = []
    K = 2 if shape == "even" else 3
    first = K * nw
    fed = ntiles >= FEED_MIN_TILES * nw

    def warp(w):
        g = w % ng
        st = {"more": fed and first + g * chunk < ntiles, "pend": None}
        if st["more"]:
            st["pend"] = counters[g]
            counters[g] += 1
            yield

        def after(last):
            if last >= ntiles:
                return ntiles
            if not fed:
                return last + nw if last + nw < ntiles else ntiles
            if not st["more"]:
                return ntiles
            v = st["pend"]
            t = first + ((v // chunk) * ng + g) * chunk + v % chunk
            if t >= ntiles:
                st["more"] = False
                return ntiles
            st["pend"] = counters[g]
            counters[g] += 1
            return t

        def clip(x):
            return x if x < ntiles else ntiles

        t = w
        if t < ntiles:
            if shape == "even":
                t1 = clip(w + nw)
                while True:
                    got.append(t)
                    yield
                    if t1 >= ntiles:
                        break
                    t, t1 = t1, after(t1)
                    yield
            elif shape == "odd":
                t1, t2 = clip(w + nw), clip(w + 2 * nw)
                while True:
                    t3 = after(t2)
                    yield
                    got.append(t)
                    yield
                    if t1 >= ntiles:
                        break
                    t, t1, t2 = t1, t2, t3
            else:
                t1, t2 = clip(w + nw), clip(w + 2 * nw)
                while True:
                    got.append(t)
                    yield
                    if t1 >= ntiles:
                        break
                    t, t1, t2 = t1, t2, after(t2)
                    yield
        assert not st["more"], "a taken counter value was left unused"
        # feed_done: the block's last warp past its barrier counts the block
        b = w // warps_per_block
        done_warps[b] += 1
        if fed and done_warps[b] == warps_per_block:
            counters[ng] += 1
            if counters[ng] == nblocks:
                counters[:] = [0] * (ng + 1)
        yield

    gens = [warp(w) for w in range(nw)]
    live = list(range(nw))
    while live:
        i = rng.choice(live)
        try:
            next(gens[i])
        except StopIteration:
            live.remove(i)
    assert sorted(got) == list(range(ntiles))
    assert counters == [0] * (ng + 1)
    return fed


@pytest.mark.parametrize("shape", ["even", "odd", "dense"])
@pytest.mark.parametrize("groups,chunk", [(1, 32), (8, 32), (8, 2), (3, 1)])
def test_every_tile_once_and_counters_rearmed(shape, groups, chunk):
    fed_seen = set()
    for nw, wpb in ((4, 4), (8, 4), (12, 4), (16, 8)):
        for ntiles in (1, 5, nw - 1, nw, 3 * nw + 1, FEED_MIN_TILES * nw - 1, FEED_MIN_TILES * nw,
                       FEED_MIN_TILES * nw + 37, 40 * nw + 3):
            if ntiles < 1:
                continue
            for seed in range(2):
                fed_seen.add(launch(ntiles, nw, shape, groups, chunk, wpb, seed))
    assert fed_seen == {True, False}
