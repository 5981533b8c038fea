"""The tile-scale request stream of bench.py's served workload, on the CPU:
every tile id serves exactly its 6 neighbours, no more than `window` tiles
are in flight at once, and the walk is reproducible from its seed."""
import collections
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def _walk(n, window, seed):
    import bench
    w = bench.TileWalk(n, window, 6, seed)
    draws, live_max = [], 0
    while True:
        d = w.draw()
        if d is None:
            break
        draws.append(d)
        live_max = max(live_max, len(w.active))
    return draws, live_max


def test_every_tile_serves_six_neighbours():
    draws, live_max = _walk(1000, 32, 7)
    per = collections.Counter(t for t, _ in draws)
    assert len(per) == 1000 and set(per.values()) == {6}
    # each tile's draws number its neighbours 0..5 in order
    seen = collections.defaultdict(list)
    for t, j in draws:
        seen[t].append(j)
    assert all(v == list(range(6)) for v in seen.values())
    assert live_max <= 32


def test_window_bounds_the_reuse_distance():
    """A tile's six uses fall within a bounded stretch of the stream: the
    cache needs only about `window` live entries per class."""
    draws, _ = _walk(500, 16, 3)
    first, last = {}, {}
    for i, (t, _) in enumerate(draws):
        first.setdefault(t, i)
        last[t] = i
    spans = sorted(last[t] - first[t] for t in first)
    assert spans[len(spans) // 2] < 16 * 6 * 2


def test_walk_is_reproducible():
    assert _walk(200, 8, 11) == _walk(200, 8, 11)
    assert _walk(200, 8, 11) != _walk(200, 8, 12)
