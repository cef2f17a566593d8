"""C ABI and host-side logic, on CPU (no kernel runs here)."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pfast_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pfast_[a-z0-9_A-Z]+)\s*\(", text)))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for ref_name in ("pfast_fsm3d", "pfast_adjoint_fsm3d", "pfast_RT_fsm2d", "pfast_Tadjoint_fsm2d",
                     "pfast_Radjoint_fsm2d", "pfast_survey3d_eval", "pfast_survey2d_eval"):
        assert ref_name in names


def test_library_exports_every_declared_symbol():
    from pfast_gb300 import _capi
    L = _capi.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    bound = {s[0] for s in _capi.SIGNATURES}
    assert bound == set(declared_functions())


def test_library_exports_only_the_c_abi():
    from pfast_gb300 import _capi
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T pfast" in l}
    assert exported == set(declared_functions())


def test_status_strings_and_version_without_gpu():
    from pfast_gb300 import _capi
    L = _capi.lib()
    assert b"sm_103a" in L.pfast_version()
    for s in range(7):
        assert L.pfast_status_string(s)


def test_context_without_device_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import pfast_gb300 as pg
    with pytest.raises(pg.PfastError) as e:
        pg.Context(0)
    assert e.value.status == 4   # PFAST_ERR_NO_DEVICE


def test_reference_shim_rejects_bad_arrays():
    import pfast_gb300 as pg
    vp = np.ones((2, 2, 2))
    with pytest.raises(TypeError):
        pg.fsm3d(vp.astype(np.float32), np.empty((2, 2, 2)), np.zeros(3, np.int32), 0, 10, 1, 1, 1, 2, 2, 2)


def test_inp_parsers_and_index_conversion(tmp_path):
    from pfast_gb300 import io as pio
    p2 = tmp_path / "a.inp"
    p2.write_text("#c\nm.vp\ns.src\n56 3\nr.rec\n33600 7\nz.ref\n1200 3\n160.000000 600.000000 12.500000 8.000000\n"
                  "out.vp\n60 20\nw.wr\n#x\n3 2\n")
    d = pio.parse_inp2d(str(p2))
    assert (d["NX"], d["NY"], d["dx"], d["dz"], d["NumofR"], d["wr"]) == (160, 600, 12.5, 8.0, 2, "w.wr")
    p3 = tmp_path / "b.inp"
    p3.write_text("a.vp\nb.src\n690 4\nc.rec\n886326 7\n150 310 200 20 20 10\nout.vp\n200 200 10\n3 2\n")
    d3 = pio.parse_inp3d(str(p3))
    assert (d3["NX"], d3["NY"], d3["NZ"], d3["dz"], d3["lsrc"]) == (150, 310, 200, 10.0, 2)
    # ceil(x/h)-1: a node at index i sits at (i+1)*h
    assert list(pio.to_index([10.0, 10.1, 19.9, 20.0], 10.0)) == [0, 1, 1, 1]


def test_synthetic_generators_are_seeded():
    from pfast_gb300 import synth
    a = synth.random_small3d((3, 4, 5), 9)
    b = synth.random_small3d((3, 4, 5), 9)
    assert np.array_equal(a, b)
    src, srnum, rec, nxyz = synth.surface_survey3d(256, 256, 16, 64)
    assert src.shape == (256, 3) and rec.shape == (256 * 4096, 3) and int(srnum.sum()) == len(rec)
    assert (src[:, 2] == 0).all() and (rec[:, 2] == 0).all()
    # no receiver sits on a source node
    s = {tuple(x) for x in src}
    assert not any(tuple(x) in s for x in rec[:4096])
    vt, v0, Z = synth.joint2d_models()
    assert vt.shape == (201, 601) and Z.shape == (601, 3)
    assert np.all(Z[:, 1] < 0)


def test_workload_generators_load_no_cuda_library():
    """bench.py's reference arm imports the seeded generators; they must not map
    libpfast_gb300.so (the reference arm runs the CPU restatement only)."""
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import pfast_gb300\n"
            "from pfast_gb300 import synth, workloads, _capi\n"
            "workloads.c3_inputs(8, 16, 16, 2, 4)\n"
            "assert _capi._lib is None\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libpfast_gb300' not in maps\n" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]


def test_option_and_stats_layout_match_the_header():
    """The ctypes mirrors of pfast_options / pfast_stats carry every field of the header's
    structs in order, and the tuner's candidate constants agree with it."""
    import ctypes as C
    from pfast_gb300 import _capi
    text = open(HEADER).read()
    for struct, cls in (("pfast_options", _capi.Options), ("pfast_stats", _capi.Stats)):
        body = re.search(r"typedef struct \{([^{}]*)\}\s*" + struct + ";", text).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        fields = [f for decl in body.split(";") if decl.strip() for f in re.findall(r"(\w+)\s*(?=,|$)", decl.strip())]
        assert fields == [name for name, _ in cls._fields_], struct
    assert int(re.search(r"#define PFAST_TUNE_CANDIDATES (\d+)", text).group(1)) == len(_capi.PFAST_TUNE_CANDIDATES)
    assert int(re.search(r"#define PFAST_SCHEDULE_HYBRID (\d+)", text).group(1)) == _capi.PFAST_SCHEDULE_HYBRID
    assert int(re.search(r"#define PFAST_TILE_8x4x32 (\d+)", text).group(1)) == _capi.PFAST_TILE_8x4x32
    assert C.sizeof(_capi.Stats) % 8 == 0


def test_phase_candidates_decoding():
    """pfast_stats.candidates: 4 bits per sweep kind, 1 + the candidate index, 0 = not run."""
    from pfast_gb300 import _capi
    # FP32 forward: per diagonal 4x8x32 (0); forward polish: persistent 4x8x32 (2); FP32 adjoint:
    # per diagonal 8x4x32 (1); adjoint polish: hybrid 4x8x32 (4); the plain kinds not run
    c = (0 + 1) << 4 | (2 + 1) << 8 | (1 + 1) << 16 | (4 + 1) << 20
    got = _capi.phase_candidates({"candidates": c})
    assert got == {"fwd32": "diagonal 4x8x32", "fwd64_polish": "persistent 4x8x32", "adj32": "diagonal 8x4x32",
                   "adj64_polish": "hybrid 4x8x32"}
    assert _capi.phase_candidates({"candidates": 0}) == {}
