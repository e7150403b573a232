"""bench.py prints its result as one JSON line of its own, also when C code
in the same process has left unflushed text in the C stdio buffer (the
library prints the reference's banners with printf, which is fully buffered
when stdout is a file or a pipe)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

CODE = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
import bench
libc = ctypes.CDLL(None)
libc.printf(b"Nx,Ny,Nz,Lx  |  ")          # a banner left without its newline
bench.emit({"metric": "m", "value": 1.5})
libc.printf(b"tail after the result\n")
"""


def test_json_line_stands_alone():
    r = subprocess.run([sys.executable, "-c", CODE, str(ROOT)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    assert json.loads(lines[0]) == {"metric": "m", "value": 1.5}
    assert "Nx,Ny,Nz,Lx" in r.stdout  # the banner is kept, on a line of its own
