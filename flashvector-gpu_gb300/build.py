"""Build recipe for libfvgb300.so (CUDA kernels + C ABI + C++ host engine).

Compiles every translation unit under csrc/ for sm_103a in parallel with
nvcc and links one shared library next to this file (in-tree, so the
process that loads it is visibly using it). Re-running is incremental:
an object is rebuilt only when its source or any header is newer.

    python flashvector-gpu_gb300/build.py [--force] [--jobs N]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "fvgb300" / "libfvgb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills", f"-I{ROOT / 'include'}", f"-I{PKG / '_build'}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


TUNING = PKG / "tuning" / "gb300.json"
TUNE_INC = OBJ / "tuning_table.inc"
TUNE_IVF_INC = OBJ / "tuning_ivf.inc"
IVF_MODES = {"pq": 0, "sq8": 1, "rabitq": 2}
METRICS = {"l2": 0, "cosine": 1, "ip": 2}


def _tuning_table() -> None:
    """tuning/gb300.json (committed autotuner results) -> _build/tuning_table.inc,
    one TuneEntry initialiser per entry (see csrc/tc_scan.cu)."""
    import json

    lines = []
    if TUNING.exists():
        for e in json.loads(TUNING.read_text()).get("entries", []):
            k = e["knobs"]
            lines.append("    {%d, %d, %du, %du, %dull, %dull, %du, %du, %du, %du, %d, %d, %d, %d},"
                         % (1 if e["precision"] == "fp8" else 0, METRICS[e["metric"]], e["dim"][0], e["dim"][1],
                            e["n"][0], e["n"][1], e["nq"][0], e["nq"][1], e["k"][0], e["k"][1], k.get("pair", -1),
                            k.get("prepass", -1), k.get("stride", 0), k.get("overfetch", 0)))
    text = "// generated by build.py from tuning/gb300.json\n" + "\n".join(lines) + ("\n" if lines else "")
    if not TUNE_INC.exists() or TUNE_INC.read_text() != text:
        TUNE_INC.write_text(text)
    # IVF entries: one IvfTuneEntry initialiser each (see csrc/ivf.cu)
    lines = []
    if TUNING.exists():
        for e in json.loads(TUNING.read_text()).get("ivf_entries", []):
            k = e["knobs"]
            lines.append("    {%d, %du, %du, %dull, %dull, %du, %du, %du, %du, %du, %du, %d, %d, %d},"
                         % (IVF_MODES[e["mode"]], e["dim"][0], e["dim"][1], e["n"][0], e["n"][1], e["nlist"][0],
                            e["nlist"][1], e["nq"][0], e["nq"][1], e["nprobe"][0], e["nprobe"][1],
                            k.get("pipeline", -1), k.get("split", -1), k.get("tc_coarse", -1)))
    text = "// generated by build.py from tuning/gb300.json\n" + "\n".join(lines) + ("\n" if lines else "")
    if not TUNE_IVF_INC.exists() or TUNE_IVF_INC.read_text() != text:
        TUNE_IVF_INC.write_text(text)


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")) + [TUNE_INC, TUNE_IVF_INC]


def _stale(src: Path, obj: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    _tuning_table()
    nvcc = _nvcc()
    newest = max((h.stat().st_mtime for h in _headers()), default=0.0)
    cmds = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(src, obj, newest):
            cmds.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.stem + ".cpp.o")
        objs.append(obj)
        if force or _stale(src, obj, newest):
            cmds.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stderr.strip()):
            print(r.stderr, flush=True)
        return r

    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(run, cmds))
    if force or cmds or not LIB.exists():
        link = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp"]
        run(link)
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.jobs, verbose=a.verbose))


if __name__ == "__main__":
    sys.exit(main())
