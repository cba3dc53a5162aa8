"""The default bench line's side workloads, on the CPU: each runs in a
child process whose JSON line is read back, and a child that fails or prints
no line leaves an error string in place of its summary (the main line is
still printed)."""
import importlib
import sys
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
bench = importlib.import_module("bench")


def test_json_lines_keeps_only_json_objects():
    text = 'building...\n{"a": 1}\nnot json {\n{"b": [1, 2]}\n{broken\n'
    assert bench._json_lines(text) == [{"a": 1}, {"b": [1, 2]}]


def test_child_returns_its_lines():
    lines, err, wall = bench._child(["-c", 'print("log"); print(\'{"value": 3}\')'], 60)
    assert err is None and lines == [{"value": 3}] and wall >= 0


def test_child_failure_is_an_error_string():
    lines, err, _ = bench._child(["-c", "import sys; sys.stderr.write('boom\\n'); sys.exit(3)"], 60)
    assert lines is None and err.startswith("exit 3") and "boom" in err
    lines, err, _ = bench._child(["-c", "print('no json here')"], 60)
    assert lines is None and err.startswith("exit 0")
