"""Writes tests/golden/ls_rounds_regression_1m.txt.gz: the local-search
candidates of the eight intermediate models of the 1M-row, 5-feature
regression search (rils_rols_gb300.synth.REGRESSION_1M_TRAJECTORY), one line
per candidate, "<round>\\t<prefix tree>", rounds in order.

The candidates come from the reference's own all_candidates
(rils_rols_cpp.cpp:348-443) through the reference harness
(oracle/_ref/librr_ref.so, built by oracle/build_ref.sh where the reference
checkout exists), so that the CPU baseline can score the benchmark's
candidates without the product library.  The product's generator must give
the same lists (tests/test_workload_cpu.py checks it).

    python tests/golden/make_workload.py [REFERENCE_ROOT]
"""
import ctypes as C
import gzip
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "rils-rols_gb300"))
from rils_rols_gb300 import synth  # noqa: E402

OUT = HERE / "ls_rounds_regression_1m.txt.gz"


def main():
    subprocess.run([str(REPO / "oracle" / "build_ref.sh")] + sys.argv[1:2], check=True)
    lib = C.CDLL(str(REPO / "oracle" / "_ref" / "librr_ref.so"))
    buf = C.create_string_buffer(1 << 24)
    lines = []
    for r, model in enumerate(synth.REGRESSION_1M_TRAJECTORY):
        n = lib.ref_candidates(model.encode(), 1, 5, 0, buf, len(buf))
        if n < 0:
            raise RuntimeError(buf.value[:300])
        for line in buf.value.decode().split("\n"):
            if line:
                lines.append(f"{r}\t{line.split(chr(9))[1]}")
    # mtime 0: the same bytes on every run
    with gzip.GzipFile(OUT, "wb", mtime=0) as f:
        f.write(("\n".join(lines) + "\n").encode())
    print(OUT, len(lines), "candidates")


if __name__ == "__main__":
    main()
