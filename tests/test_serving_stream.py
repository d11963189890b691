"""The serving job stream: seeded, 70/25/5 % by size class, supports within
[1 %, 5 %] of n, k by class."""
import collections


def test_stream_shape():
    from gspan_gb300 import datagen
    classes = [0] * 8 + [1] * 3 + [2]
    sizes = [3300] * 8 + [100000] * 3 + [3700000]
    jobs = datagen.serving_jobs(classes, sizes, 4000, rate=50.0, seed=7)
    assert jobs == datagen.serving_jobs(classes, sizes, 4000, rate=50.0, seed=7)
    times = [t for t, *_ in jobs]
    assert times == sorted(times)
    assert abs(len(jobs) / times[-1] - 50.0) < 5.0
    cnt = collections.Counter(classes[gi] for _, gi, _, _ in jobs)
    for c, share in enumerate(datagen.SERVING_MIX):
        assert abs(cnt[c] / len(jobs) - share) < 0.03
    for _, gi, k, sup in jobs:
        assert int(0.01 * sizes[gi]) <= sup <= 0.05 * sizes[gi]
        assert k in ((3, 4) if classes[gi] == 0 else (3,))
