"""The C-ABI library without a GPU: layout, exports, numbering, validation.

Mirrors the device-free parts of the reference's abi_smoke.c
(corr-cuda/tests/abi_smoke.c:62-141) and the Rust layout asserts
(corr-rs/src/ffi.rs). Nothing here launches a kernel.
"""

from __future__ import annotations

import ctypes as C
import re
import subprocess
import threading
from pathlib import Path

import pytest

from conftest import REPO

INCLUDE = REPO / "include"


def declared_functions() -> set[str]:
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(corr\w*)\s*\(", text, re.M):
            names.add(m.group(1))
    names.discard("corr_notify_fn")
    return names


def test_every_declared_symbol_is_exported(pkg):
    lib_path = pkg.abi.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    declared = declared_functions()
    assert len(declared) >= 32
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    # and the ctypes binding table covers exactly the declarations
    assert declared == set(pkg.abi.SIGNATURES)


def test_struct_layouts_match_header(pkg, tmp_path):
    """Compile the header with gcc and compare sizeof/offsetof with the ctypes mirror."""
    src = tmp_path / "layout.c"
    fields = {
        "corr_config": [f for f, _ in pkg.abi.corr_config._fields_],
        "corr_device_plan": [f for f, _ in pkg.abi.corr_device_plan._fields_],
        "corr_device_stats": [f for f, _ in pkg.abi.corr_device_stats._fields_],
        "corr_staging": [f for f, _ in pkg.abi.corr_staging._fields_],
        "corrx_params": [f for f, _ in pkg.abi.corrx_params._fields_],
        "corrx_tiles": [f for f, _ in pkg.abi.corrx_tiles._fields_],
        "corrx_frontend": [f for f, _ in pkg.abi.corrx_frontend._fields_],
        "corrx_tc_geom": [f for f, _ in pkg.abi.corrx_tc_geom._fields_],
        "corrw_station": [f for f, _ in pkg.abi.corrw_station._fields_],
        "corrw_params": [f for f, _ in pkg.abi.corrw_params._fields_],
        "corrw_resume": [f for f, _ in pkg.abi.corrw_resume._fields_],
        "corrw_stats": [f for f, _ in pkg.abi.corrw_stats._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "corr_gb300.h"',
             '#include "corr_writer.h"',
             "int main(void) {"]
    for s, fl in fields.items():
        lines.append(f'printf("{s} size %zu\\n", sizeof({s}));')
        for f in fl:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-I", str(INCLUDE), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.splitlines())
    for s, fl in fields.items():
        cls = getattr(pkg.abi, s)
        assert int(got[f"{s} size"]) == C.sizeof(cls), s
        for f in fl:
            assert int(got[f"{s}.{f}"]) == getattr(cls, f).offset, f"{s}.{f}"
    # the reference's byte sizes (corr-rs/src/ffi.rs layout asserts)
    assert int(got["corr_config size"]) == 76
    assert int(got["corr_staging size"]) == 48
    assert int(got["corr_device_plan size"]) == 20
    assert int(got["corr_device_stats size"]) == 72


def test_c_caller_compiles_and_links(pkg, tmp_path):
    """A plain C program written against the header links against the .so."""
    src = tmp_path / "caller.c"
    src.write_text("""
#include <stdio.h>
#include <string.h>
#include "corr_cuda.h"
int main(void) {
    printf("%s\\n", corr_abi_banner());
    return corr_n_baseline(24) == 300 ? 0 : 1;
}
""")
    exe = tmp_path / "caller"
    libdir = pkg.abi.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c99", "-I", str(INCLUDE), str(src), "-L", str(libdir),
                    "-lcorr_cuda", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0
    assert "abi=7" in res.stdout


def test_banner_and_error_string(lib):
    banner = lib.corr_abi_banner().decode()
    assert "abi=7" in banner and "sm_103a" in banner
    seen = {}

    def fresh_thread():
        seen["err"] = lib.corr_last_error()
    t = threading.Thread(target=fresh_thread)
    t.start()
    t.join()
    assert seen["err"] == b""          # thread-local, starts empty
    st = lib.corr_create(None, None)
    assert st == 1                      # CORR_ERR_ARG
    assert len(lib.corr_last_error()) > 0


def test_baseline_numbering(pkg, lib, oracle):
    assert lib.corr_n_baseline(0) == -1
    assert lib.corr_n_baseline(1) == 1
    assert lib.corr_n_baseline(4) == 10
    assert lib.corr_n_baseline(15) == 120
    assert lib.corr_n_baseline(24) == 300
    assert lib.corr_n_baseline(40) == 820
    for n in range(1, 45):
        assert pkg.Correlator.baseline_pairs(n) == oracle.baseline_pairs(n)
    arr = (C.c_int32 * 19)()
    assert lib.corr_baseline_pairs(4, arr, 19) == 1
    assert lib.corr_baseline_pairs(0, arr, 0) == 1


def _cfg(pkg, **kw):
    base = dict(n_station=4, n_freq=4096, frames_per_slot=16, chunk_frames=8, block_slots=3,
                rows_per_fetch=2)
    base.update({k: v for k, v in kw.items() if k in base})
    cfg = pkg.make_config(**base)
    for k, v in kw.items():
        if k not in base:
            setattr(cfg, k, v)
    return cfg


@pytest.mark.parametrize("change,status", [
    (dict(abi_version=8), 2),              # CORR_ERR_ABI
    (dict(struct_size=72), 2),
    (dict(n_freq=4096 + 1024), 1),         # not a power of two / multiple of 2048
    (dict(n_freq=34816), 8),               # multiple of 2048 above 32768: NOT_IMPL
    (dict(n_freq=3072), 1),                # neither a power of two nor a multiple of 2048
    (dict(n_freq=256), 1),
    (dict(n_freq=65536), 8),
    (dict(block_slots=1), 1),
    (dict(chunk_frames=17), 1),            # > frames_per_slot
    (dict(chunk_frames=0), 1),
    (dict(frames_per_slot=0, chunk_frames=0), 1),
    (dict(rows_per_fetch=0), 1),
    (dict(n_station=0), 1),
    (dict(n_station=45), 1),               # 1035 baselines > 1024
    (dict(n_devices=9), 1),
    (dict(n_devices=-1), 1),
    (dict(split_mode=3), 1),
    (dict(device_id=-1), 1),
])
def test_config_rejection(pkg, lib, change, status):
    cfg = _cfg(pkg, **change)
    ctx = C.c_void_p(0x1)
    st = lib.corr_create(C.byref(cfg), C.byref(ctx))
    assert st == status, lib.corr_last_error()
    assert ctx.value is None
    assert len(lib.corr_last_error()) > 0


def test_create_without_gpu_reports_cuda_error(pkg, lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    st = lib.corr_create(C.byref(_cfg(pkg)), C.byref(ctx))
    assert st == 3  # CORR_ERR_CUDA: no device to talk to
    assert ctx.value is None


def test_null_context_calls(lib):
    out = C.c_int32()
    assert lib.corr_destroy(None) == 0
    assert lib.corr_row_accumulate(None, 0, 1) == 1
    assert lib.corr_row_slot_free(None, 0) == 1
    assert lib.corr_row_end(None, 1) == 1
    assert lib.corr_rows_pending(None, C.byref(out)) == 1
    assert lib.corr_n_devices(None) == -1
    assert lib.corrx_accumulate(None, None, 0, 0, None, 0, 0, 0, None, None) == 1
    assert lib.corrx_accumulate_packets(None, None, 0, 0, None, 0, 0, None, 0, 0, 0, None,
                                        None) == 1
