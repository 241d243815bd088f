"""The bench's reference arm on the CPU: `bench.py --impl reference` times the
oracle (the reference's algorithm restated in C) on a sample of the workload
and prints the contract's JSON line, loading nothing of the library -- no
build, no liborgpu.so -- so that its number stands apart from the product."""
import io
import json
import os
import sys
from contextlib import redirect_stdout

from conftest import REPO


def test_reference_arm_runs_the_oracle_only(monkeypatch):
    sys.path.insert(0, REPO)
    import bench
    from orgpu import _lib
    loaded_before = _lib._lib
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                                      "--events", "300", "--cpu-sample", "300", "--no-reference-gpu"])
    out = io.StringIO()
    with redirect_stdout(out):
        bench.main()
    line = json.loads([l for l in out.getvalue().splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "events/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    # the library was neither loaded by this arm nor mapped into the process by it
    if loaded_before is None:
        assert _lib._lib is None
        maps = open("/proc/self/maps").read() if os.path.exists("/proc/self/maps") else ""
        assert "liborgpu" not in maps
