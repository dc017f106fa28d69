"""The build recipe targets sm_103a alone and builds the same on x86_64 and
aarch64 hosts: no host-ISA flags, no ISA-specific intrinsics headers or host
inline assembly, and the oracle's Makefile likewise.  No compiler is run."""
from __future__ import annotations

import importlib.util
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "bale_old_gb300" / "csrc"


def _build_module():
    spec = importlib.util.spec_from_file_location("bale_build", ROOT / "bale_old_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_nvcc_targets_sm_103a_only():
    b = _build_module()
    flags = b.NVCC_FLAGS
    gencodes = [flags[i + 1] for i, f in enumerate(flags) if f == "-gencode"]
    assert gencodes == ["arch=compute_103a,code=sm_103a"]
    assert not any(f.startswith(("-arch", "--gpu-architecture", "-code")) for f in flags)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_no_host_isa_flags():
    b = _build_module()
    host_flags = list(b.CC_FLAGS) + [f for f in b.NVCC_FLAGS if f.startswith("-m") or "march" in f]
    assert not [f for f in host_flags if re.match(r"-m(arch|tune|cpu|avx|sse|fma|bmi|64$|32$)", f)], host_flags
    makefile = (ROOT / "oracle" / "Makefile").read_text()
    assert not re.search(r"-m(arch|tune|cpu|avx|sse)", makefile)


def _sources():
    pats = ("*.cu", "*.cuh", "*.c", "*.h")
    out = [p for pat in pats for p in CSRC.rglob(pat)]
    out += [p for pat in ("*.c", "*.h") for p in (ROOT / "oracle").glob(pat)]
    out += list((ROOT / "include").glob("*.h"))
    return sorted(set(out))


def test_no_isa_specific_host_headers():
    bad = re.compile(r'#\s*include\s*<(immintrin|xmmintrin|emmintrin|pmmintrin|smmintrin|nmmintrin|'
                     r'x86intrin|cpuid|arm_neon|arm_sve)\.h>')
    hits = [p.name for p in _sources() if bad.search(p.read_text())]
    assert not hits, hits


def test_host_c_has_no_inline_assembly():
    # inline PTX lives in the .cu/.cuh device code; the host C files carry none
    hosts = [p for p in _sources() if p.suffix in (".c", ".h")]
    hits = [p.name for p in hosts if re.search(r"\b(__asm__|asm)\s*(volatile\s*)?\(", p.read_text())]
    assert not hits, hits


def test_every_cuda_source_is_built():
    b = _build_module()
    assert b.CSRC == CSRC
    cu = sorted(p.name for p in CSRC.glob("*.cu"))
    assert {"capi.cu", "histo.cu", "ig.cu", "ig_part.cu", "triangle.cu", "tri_wedge.cu",
            "tri_hybrid.cu", "batch.cu", "serve.cu"} <= set(cu)
    # the recipe globs csrc/*.cu: nothing with CUDA code sits deeper down
    assert not [p for p in CSRC.rglob("*.cu") if p.parent != CSRC]
