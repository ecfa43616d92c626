"""The benchmark line's legs after the headline report their own failures.

bench.py runs the configuration, batched-form, median-filter, omnical and
serving legs after the headline; a leg that raises (a library error, a
device-side wait that gave up) puts its error into its own object and the
line is still printed.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_a_working_leg_returns_its_result():
    assert bench.run_leg(lambda a, b: {"sum": a + b}, 2, 3) == {"sum": 5}


def test_a_failing_leg_reports_its_error(capsys):
    def leg():
        raise RuntimeError("a device-side wait gave up")

    out = bench.run_leg(leg)
    assert out == {"error": "RuntimeError: a device-side wait gave up"}
    assert "Traceback" in capsys.readouterr().err
