"""The C-ABI library loads and exports every entry point declared in
include/*.h (no compute calls: no GPU needed)."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:pg_status|void|const char\s*\*)\s*(pg_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_abi():
    from pilon_gb300 import _abi
    assert declared() == set(_abi.EXPORTED)


def test_library_exports_every_declared_symbol():
    from pilon_gb300.build import ENGINE, build
    if not os.path.exists(ENGINE):
        build()
    lib = C.CDLL(ENGINE)
    for name in declared():
        assert hasattr(lib, name), name


def test_struct_layouts_match_header():
    from pilon_gb300 import _abi
    # sizes fixed by the header's field order (LP64)
    assert C.sizeof(_abi.pg_params) == 12 * 4 + 8  # 12 int32, then the double at offset 48
    assert C.sizeof(_abi.pg_reads) == 8 + 15 * 8 + 3 * 8
    assert C.sizeof(_abi.pg_region) == 32
    assert C.sizeof(_abi.pg_kmer_edge) == 32
    assert C.sizeof(_abi.pg_window) == 16
    assert C.sizeof(_abi.pg_break) == 16
    assert C.sizeof(_abi.pg_request) == 16
    assert C.sizeof(_abi.pg_serve_config) == 48  # 4 + 4, the int64 budget at 8, then 7 int32 + padding
    assert C.sizeof(_abi.pg_result) == 96
    assert _abi.pg_result.latency_ms.offset == 80 and _abi.pg_serve_config.hbm_budget.offset == 8
    assert C.sizeof(_abi.pg_reassembly) == 10 * 4 + 2 * 8 and _abi.pg_reassembly.bases.offset == 40
    assert C.sizeof(_abi.pg_reassembly_fix) == 4 * 4 + 4 * 8 and _abi.pg_reassembly_fix.patch_off.offset == 32


def test_default_params_match_pilon():
    from pilon_gb300 import _abi
    from pilon_gb300.build import ENGINE, build
    if not os.path.exists(ENGINE):
        build()
    lib = C.CDLL(ENGINE)
    p = _abi.pg_params()
    lib.pg_default_params(C.byref(p))
    q = _abi.default_params()
    for f, _ in _abi.pg_params._fields_:
        assert getattr(p, f) == getattr(q, f), f


def test_open_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pilon_gb300.engine import Engine, EngineError
    with pytest.raises(EngineError):
        Engine(0)


def _lib():
    from pilon_gb300.build import ENGINE, build
    if not os.path.exists(ENGINE):
        build()
    lib = C.CDLL(ENGINE)
    lib.pg_last_error.restype = C.c_char_p
    lib.pg_last_error.argtypes = [C.c_void_p]
    lib.pg_close.argtypes = [C.c_void_p]
    return lib


def test_open_errors_are_statuses():
    """pg_open with a NULL out pointer, a negative device, or no device at all
    returns a status and a message; a context that failed to open refuses the
    device calls with PG_ERR_STATE and closes cleanly."""
    from pilon_gb300 import _abi
    lib = _lib()
    assert lib.pg_open(None, 0) == _abi.PG_ERR_ARG
    bad = C.c_void_p()
    assert lib.pg_open(C.byref(bad), -1) == _abi.PG_ERR_CUDA
    assert lib.pg_last_error(bad) == b"no CUDA device -1"
    lens = (C.c_int64 * 1)(4)
    base = (C.c_uint8 * 4)(*b"ACGT")
    bases = (C.c_void_p * 1)(C.addressof(base))
    long_lens = (C.c_int64 * 1)(2 ** 31)
    assert lib.pg_set_reference(bad, 1, long_lens, bases) == _abi.PG_ERR_ARG
    assert lib.pg_last_error(bad) == b"contig 0 is longer than 2^31 - 1 bases"
    assert lib.pg_set_reference(bad, 1, lens, bases) == _abi.PG_ERR_STATE
    assert lib.pg_last_error(bad) == b"the context is not open (pg_open failed: no CUDA device -1)"
    assert lib.pg_sync(bad) == _abi.PG_ERR_STATE
    reads = _abi.pg_reads()
    reads.seq_bytes = -1
    assert lib.pg_set_reads(bad, C.byref(reads)) == _abi.PG_ERR_ARG
    assert lib.pg_set_reads_device(bad, C.byref(reads)) == _abi.PG_ERR_ARG
    assert lib.pg_set_reads_packed(bad, C.byref(reads)) == _abi.PG_ERR_ARG
    assert lib.pg_last_error(bad) == b"negative array length in the read store"
    reads.seq_bytes = 0
    assert lib.pg_set_reads_packed(bad, C.byref(reads)) == _abi.PG_ERR_STATE
    assert lib.pg_set_reads(bad, C.byref(reads)) == _abi.PG_ERR_STATE
    assert lib.pg_set_reads_device(bad, C.byref(reads)) == _abi.PG_ERR_STATE
    p = _abi.default_params()
    assert lib.pg_pileup_regions(bad, None, 0, C.byref(p), 1) == _abi.PG_ERR_STATE
    stats = _abi.pg_region_stats()
    assert lib.pg_fetch_stats(bad, 0, C.byref(stats)) == _abi.PG_ERR_STATE
    # --defaultqual is a Byte in Pilon: values outside -128..127 are argument errors
    n1, n2 = C.c_int64(), C.c_int64()
    for dq, want in [(128, _abi.PG_ERR_ARG), (-129, _abi.PG_ERR_ARG), (2 ** 21, _abi.PG_ERR_ARG),
                     (127, _abi.PG_ERR_STATE), (-128, _abi.PG_ERR_STATE)]:
        q = _abi.default_params(default_qual=dq)
        assert lib.pg_pileup_regions(bad, None, 0, C.byref(q), 1) == want, dq
        assert lib.pg_kmer_tally(bad, None, 0, 31, C.byref(q), 5, None, C.c_int64(0), C.byref(n1)) == want, dq
        assert lib.pg_kmer_tally_breaks(bad, 5, 100, 31, C.byref(q), 5, None, C.c_int64(0), C.byref(n1),
                                        C.byref(n2)) == want, dq
    assert lib.pg_last_error(bad) == b"no pileup results: call pg_pileup_regions first"
    lib.pg_close(bad)

    ctx = C.c_void_p()
    st = lib.pg_open(C.byref(ctx), 0)
    if st == _abi.PG_OK:
        lib.pg_close(ctx)
        pytest.skip("a CUDA device is present")
    assert st == _abi.PG_ERR_CUDA and lib.pg_last_error(ctx) == b"no CUDA device 0"
    lib.pg_close(ctx)


C_CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "pilon_gb300.h"

int main(void) {
  pg_params p;
  pg_default_params(&p);
  if (p.flank != 10 || p.default_qual != 10 || p.min_min_depth != 5) return 2;
  pg_ctx *ctx = NULL;
  pg_status st = pg_open(&ctx, -1);
  if (st != PG_ERR_CUDA || ctx == NULL) return 3;
  if (strcmp(pg_last_error(ctx), "no CUDA device -1") != 0) return 4;
  if (pg_sync(ctx) != PG_ERR_STATE) return 5;
  pg_close(ctx);
  /* local reassembly needs no context: an empty batch of jobs */
  int64_t text_len = -1;
  if (pg_reassemble(NULL, 0, 47, NULL, 0, 1, NULL, NULL, 0, &text_len) != PG_OK || text_len != 0) return 6;
  printf("%s|%zu|%zu|%zu|%zu|%zu\n", pg_version(), sizeof(pg_region), sizeof(pg_params), sizeof(pg_kmer_edge),
         sizeof(pg_reassembly), sizeof(pg_reassembly_fix));
  return 0;
}
"""


def test_header_compiles_as_c99_and_links(tmp_path):
    """A C client (what a JNI glue file is) compiles against the header with
    -std=c99 -Wall -Werror, links the library and calls it."""
    import shutil
    import subprocess
    from pilon_gb300.build import ENGINE, build
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    if not os.path.exists(ENGINE):
        build()
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    lib_dir = os.path.dirname(ENGINE)
    lib_name = os.path.basename(ENGINE)[3:-3]  # libX.so -> X
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", lib_dir, "-l" + lib_name, "-Wl,-rpath," + lib_dir],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    version, r, p, e, j, f = out.stdout.strip().split("|")
    assert version.startswith("pilon_gb300") and (int(r), int(p), int(e), int(j), int(f)) == (32, 56, 32, 56, 48)


C_NOMEM_CLIENT = r"""
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/resource.h>
#include <unistd.h>
#include "pilon_gb300.h"

int main(void) {
  /* one window of 2^21 edges: its graph table needs about 150 MB of host memory */
  const int64_t n_edges = (int64_t)1 << 21;
  pg_kmer_edge_wide *edges = calloc((size_t)n_edges, sizeof *edges);
  char *bases = malloc(100), *orig = malloc(100), *text = malloc(4096);
  if (!edges || !bases || !orig || !text) return 2;
  memset(edges, 0, (size_t)n_edges * sizeof *edges);
  memset(bases, 'A', 100);
  memcpy(orig, bases, 100);
  pg_reassembly job = {0, 0, 1, 100, 40, 60, 50, 0, 100000, 10, bases, orig};
  pg_reassembly_fix fix;
  int64_t text_len = -1;
  /* room for the call's own bookkeeping (about 20 MB), not for the graph */
  long vm_pages = 0;
  FILE *f = fopen("/proc/self/statm", "r");
  if (!f || fscanf(f, "%ld", &vm_pages) != 1) return 3;
  fclose(f);
  struct rlimit rl;
  rl.rlim_cur = rl.rlim_max = (rlim_t)vm_pages * (rlim_t)sysconf(_SC_PAGESIZE) + ((rlim_t)48 << 20);
  if (setrlimit(RLIMIT_AS, &rl) != 0) return 4;
  pg_status st = pg_reassemble(edges, n_edges, 31, &job, 1, 1, &fix, text, 4096, &text_len);
  printf("%d|%d\n", (int)st, (int)fix.status);
  return 0;
}
"""


def test_reassemble_host_memory_exhaustion_is_a_status(tmp_path):
    """A host allocation that fails inside pg_reassemble comes back as
    PG_ERR_NOMEM, for the call and the job, instead of a C++ exception that
    would end the caller's process (run in a child with a capped address
    space)."""
    import shutil
    import subprocess
    from pilon_gb300 import _abi
    from pilon_gb300.build import ENGINE, build
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    if not os.path.exists(ENGINE):
        build()
    src = tmp_path / "nomem.c"
    src.write_text(C_NOMEM_CLIENT)
    exe = tmp_path / "nomem"
    lib_dir = os.path.dirname(ENGINE)
    lib_name = os.path.basename(ENGINE)[3:-3]
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe), "-L", lib_dir, "-l" + lib_name, "-Wl,-rpath," + lib_dir], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    st, job = (int(x) for x in out.stdout.strip().split("|"))
    assert st == _abi.PG_ERR_NOMEM and job == _abi.PG_ERR_NOMEM
