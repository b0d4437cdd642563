"""The scatter's access-pattern probe (qpeps_probe_append; no reference
counterpart): every mode runs and times a small case, and bad arguments fail
with the library's error codes."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_every_probe_mode_times_a_small_case(ctx, qp):
    for mode in (qp.PROBE_APPEND, qp.PROBE_STORE, qp.PROBE_ATOMIC, qp.PROBE_STREAM, qp.PROBE_APPEND_PLAIN):
        ms = ctx.probe_append(mode, 1 << 20, 700, repeats=2)
        assert 0 < ms < 1000


def test_probe_rejects_bad_arguments(ctx, qp):
    with pytest.raises(qp.ContractionError) as e:
        ctx.probe_append(5, 1 << 10, 10)
    assert e.value.code == qp.QPEPS_ERR_INVALID
    with pytest.raises(qp.ContractionError) as e:
        ctx.probe_append(qp.PROBE_APPEND, 1 << 10, 0)
    assert e.value.code == qp.QPEPS_ERR_INVALID
