"""The C-ABI library loads without a GPU and exports every symbol that
include/*.h declares; sparsemat_t has the reference's layout.  No compute."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", text):
            name = m.group(1)
            if name not in {"if", "while", "for", "return", "sizeof"}:
                names.add(name)
    return names


def test_headers_declare_the_reference_entry_points():
    names = declared_functions()
    for ref in ("histo_agi", "histo_exstack", "histo_exstack2", "histo_conveyor",
                "ig_agi", "ig_exstack", "ig_exstack2", "ig_conveyor",
                "triangle_agi", "triangle_exstack_push", "triangle_exstack2_push",
                "triangle_convey_push", "triangle_agi_iter"):
        assert ref in names


def test_library_exports_every_declared_symbol():
    from bale_old_gb300._lib import LIB_PATH, SIGNATURES

    lib = C.CDLL(str(LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    # the Python binding declares a signature for every exported entry point
    assert not (declared_functions() - set(SIGNATURES)), declared_functions() - set(SIGNATURES)


def test_sparsemat_layout_matches_reference():
    from bale_old_gb300._lib import sparsemat_t

    # spmat/spmat.h:73-86: six int64 fields then four pointers
    assert C.sizeof(sparsemat_t) == 6 * 8 + 4 * 8
    assert sparsemat_t.loffset.offset == 7 * 8
    assert sparsemat_t.lnonzero.offset == 9 * 8


def test_version_and_error_calls_need_no_gpu(bale):
    assert "sm_103a" in bale.version()
    assert isinstance(bale._last_error(), str)


def test_random_permutations_follow_the_reference_seed_rule_on_empty_input(bale):
    """The reference calls srand48(seed) for a seed whose low 32 bits (its
    int) are nonzero and otherwise continues the C library's drand48 stream
    (spmat_agi.upc:61, spmat_exstack.upc:92), even when it then draws
    nothing.  With n = 0 the entry points do no device work, so this runs
    without a GPU: the next lrand48() shows the stream they left."""
    from bale_old_gb300._lib import _lib

    libc = C.CDLL(None)
    libc.srand48.argtypes = [C.c_long]
    libc.lrand48.restype = C.c_long

    def next_after(call, start):
        libc.srand48(start)
        assert call() == 0
        return libc.lrand48()

    for call in (lambda s: (lambda: _lib.bale_rand_perm_dev(0, s, None, None)),
                 lambda s: (lambda: _lib.bale_rand_perm_exstack_dev(0, s, 1024, None, None)),
                 lambda s: (lambda: _lib.bale_rand_perm_exstack2_dev(0, s, 1024, None, None))):
        for seed in (0, 1 << 32, 7 << 32):  # low 32 bits 0: the stream continues
            libc.srand48(99)
            want = libc.lrand48()
            assert next_after(call(seed), 99) == want
        libc.srand48(12345)
        want = libc.lrand48()
        assert next_after(call(12345), 99) == want  # reseeded with 12345
        assert next_after(call((5 << 32) + 12345), 99) == want  # only the low 32 bits count


def test_a_c_program_compiles_links_and_runs_against_the_library(tmp_path):
    """What an app does: include the headers as strict C, link
    libbale_gb300.so in place of the reference kernels, and resolve every
    drop-in.  The program only calls bale_version(), which needs no GPU."""
    import shutil
    import subprocess

    from bale_old_gb300._lib import LIB_PATH

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest

        pytest.skip("no C compiler")
    src = tmp_path / "app.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "bale_gb300.h"
#include "bale_inputs.h"
typedef void (*any_fn)(void);
int main(void) {
  any_fn dropins[] = {
    (any_fn)histo_agi, (any_fn)histo_exstack, (any_fn)histo_exstack2, (any_fn)histo_conveyor,
    (any_fn)ig_agi, (any_fn)ig_exstack, (any_fn)ig_exstack2, (any_fn)ig_conveyor,
    (any_fn)triangle_agi, (any_fn)triangle_exstack_push, (any_fn)triangle_exstack2_push,
    (any_fn)triangle_convey_push, (any_fn)triangle_agi_iter};
  for (size_t i = 0; i < sizeof dropins / sizeof dropins[0]; i++)
    if (!dropins[i]) return 2;
  if (sizeof(sparsemat_t) != 80) return 3;
  printf("%s\n", bale_version());
  return strstr(bale_version(), "sm_103a") ? 0 : 4;
}
''')
    exe = tmp_path / "app"
    lib_dir = LIB_PATH.parent
    build = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
                            "-o", str(exe), f"-L{lib_dir}", "-lbale_gb300", f"-Wl,-rpath,{lib_dir}"],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    assert "sm_103a" in run.stdout


def test_binding_signatures_match_the_header_prototypes():
    """Each ctypes signature has as many parameters as the C prototype it
    binds, and pointer-ness agrees parameter by parameter."""
    from bale_old_gb300._lib import SIGNATURES

    protos = {}
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}()]*)\)\s*;", text):
            params = [p.strip() for p in m.group(2).replace("\n", " ").split(",") if p.strip()]
            if params == ["void"]:
                params = []
            protos[m.group(1)] = params
    bad = []
    for name, params in protos.items():
        if name not in SIGNATURES:
            continue
        argtypes = SIGNATURES[name][1]
        if len(argtypes) != len(params):
            bad.append((name, len(params), len(argtypes)))
            continue
        for p, a in zip(params, argtypes):
            c_ptr = "*" in p
            py_ptr = a is C.c_void_p or a is C.c_char_p or hasattr(a, "contents") or \
                (isinstance(a, type) and issubclass(a, C._Pointer))
            if c_ptr != py_ptr:
                bad.append((name, p, a))
    assert not bad, bad
