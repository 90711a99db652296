"""gg_gather_ceiling: the random-gather rates the pull gathers are measured
against run and report a positive rate for every source, with at least one
8-CTA cluster resident."""
import pytest

pytestmark = pytest.mark.gpu


def test_gather_ceiling_reports_every_rate(gpu):
    r = gpu.gather_ceiling()
    assert r["clusters"] >= 1 and r["cluster_sms"] == 8 * r["clusters"]
    for k in ("cluster_smem_gps", "own_smem_gps", "l2_small_gps", "l2_large_gps"):
        assert r[k] > 0.0, k
