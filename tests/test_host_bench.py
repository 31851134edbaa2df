"""bench.py's host-side helpers: a failing secondary measurement block is reported in the JSON
line instead of ending the run (the headline measured before it still prints), and the
learned-proposal forms alone get the empty-space density term."""
import os
import sys
from types import SimpleNamespace

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_guarded_passes_results_through():
    assert bench.guarded(lambda x, y=0: {"value": x + y}, 2, y=3) == {"value": 5}


def test_guarded_reports_a_failure(capsys):
    def boom():
        raise RuntimeError("no such buffer")
    out = bench.guarded(boom)
    assert out == {"error": "RuntimeError: no such buffer"}
    assert "no such buffer" in capsys.readouterr().err


def test_empty_space_decay_only_for_proposal_forms():
    args = SimpleNamespace(empty_space_decay=1e-3)
    assert bench.empty_space_decay(args, "proposal") == 1e-3
    assert bench.empty_space_decay(args, "march") == 0.0
