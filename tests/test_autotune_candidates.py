"""The autotuner's candidate lists (no GPU): every batch candidate names
band, CTA size, band axis, the two staged classes' thread counts and
whether they share one launch; the one-launch option appears exactly where
the two classes run the same thread count, and both settings of it are
timed there."""
from raytracer_3d_gb300.autotune import BATCH_CANDIDATES


def test_batch_candidates_shape():
    assert BATCH_CANDIDATES, "no batch candidates"
    for c in BATCH_CANDIDATES:
        assert len(c) == 6, c
        band, threads, sweep, persistent, slices, fused = c
        assert band > 0 and threads in (128, 256, 512, 1024) and sweep in (0, 1)
        assert persistent in (0, 128, 256, 512) and slices in (-1, 0, 256, 512)
        assert fused in (0, 1)
    assert len(set(BATCH_CANDIDATES)) == len(BATCH_CANDIDATES), "duplicate candidates"


def test_one_launch_offered_where_classes_share_threads():
    for c in BATCH_CANDIDATES:
        band, threads, sweep, persistent, slices, fused = c
        if persistent == slices and persistent > 0:
            twin = (band, threads, sweep, persistent, slices, 1 - fused)
            assert twin in BATCH_CANDIDATES, c      # both settings timed
        else:
            assert fused == 1, c                    # the flag has no effect: listed once
