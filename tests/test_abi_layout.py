"""The ctypes mirrors of the C ABI's structs have the C layout (no GPU).

Every struct of include/*.h that the Python package passes across the ABI is
compiled here with the system C compiler, and its size and the offset of each
field the Python mirror declares (same field names) must equal the mirror's.
"""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import pytest

from sicc_gb300 import _lib, devloop, engine, ingest, pipeline, server, tune

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "cuda_osd_stream_config_t": _lib.StreamConfig,
    "cuda_osd_osd_config_t": _lib.OsdConfig,
    "cuda_osd_bp_csr_config_t": _lib.BpCsrConfig,
    "cuda_osd_stream_stats_t": _lib.StreamStats,
    "sicc_engine_config_t": engine.EngineConfig,
    "sicc_engine_code_t": engine.EngineCode,
    "sicc_pipe_config_t": pipeline.PipeConfig,
    "sicc_pipe_tables_t": pipeline.PipeTables,
    "sicc_pipe_tx_tables_t": pipeline.PipeTxTables,
    "sicc_pipe_sync_t": pipeline.PipeSync,
    "sicc_ingest_config_t": ingest.IngestConfig,
    "sicc_ingest_frame_t": ingest.IngestFrame,
    "sicc_ingest_stats_t": ingest.IngestStats,
    "sicc_server_config_t": server.ServerConfig,
    "sicc_request_t": server.Request,
    "sicc_completion_t": server.Completion,
    "sicc_server_stats_t": server.ServerStats,
    "sicc_devloop_config_t": devloop.DevLoopConfig,
    "sicc_devloop_stats_t": devloop.DevLoopStats,
    "sicc_fec_shape_t": tune.FecShape,
    "sicc_tune_trial_t": tune.TuneTrial,
}


def _c_layout():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>"]
    lines += [f'#include "{h}"' for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h")]
    lines.append("int main(void) {")
    for cname, py in MIRRORS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'    printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append("    return 0;\n}")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines))
        r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    got = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    return got


def test_ctypes_mirrors_match_the_c_structs():
    c = _c_layout()
    bad = []
    for cname, py in MIRRORS.items():
        if c[(cname, "size")] != C.sizeof(py):
            bad.append(f"{cname}: size {c[(cname, 'size')]} vs ctypes {C.sizeof(py)}")
        for f in py._fields_:
            off = getattr(py, f[0]).offset
            if c[(cname, f[0])] != off:
                bad.append(f"{cname}.{f[0]}: offset {c[(cname, f[0])]} vs ctypes {off}")
    assert not bad, bad
