"""Drop-in forward executables (pfast_gb300/bin/*) run on reference-format inputs:
.inp parameter files and raw binary model / source / receiver / reflector files in
metres, written to a temporary directory.  Outputs must equal the reference's
(golden picks; the oracle for the shot gathers and the 3D picks), bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from helpers import bits_equal, load_fw

pytestmark = pytest.mark.gpu

BIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pfast_gb300", "bin")


def _write(path, arr):
    np.ascontiguousarray(arr, dtype="<f8").tofile(path)


def _inp2d(d, NX, NY, dx, dz, nsrc, nrec, rNY, gmNX):
    text = f"""# drop-in test
{d}/m.vp
{d}/m.src
{nsrc} 3
{d}/m.rec
{nrec} {rNY}
{d}/m.ref
{gmNX} 3
{NX} {NY} {dx} {dz}
{d}/out.vp
60 20
{d}/m.wr
3 2
"""
    p = os.path.join(d, "case.inp")
    open(p, "w").write(text)
    return p


def _metres2d(src, srnum, rec, nxy, dx, dz):
    srcA = np.stack([(src[:, 0] + 1) * dz, (src[:, 1] + 1) * dx, srnum.astype(float)], 1)
    recA = np.stack([(rec[:, 0] + 1) * dz, (rec[:, 1] + 1) * dx, nxy[:, 0], nxy[:, 1]], 1)
    return srcA, recA


def _run(exe, inp):
    r = subprocess.run([os.path.join(BIN, exe), inp], capture_output=True, text=True)
    return r


def test_rt_pfast2d_fw_nos_reproduces_golden_picks(tmp_path):
    g = load_fw()
    d = str(tmp_path)
    src, srnum, rec = g["src"], g["srnum"], g["rec"].astype(np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    srcA, recA = _metres2d(src, srnum, rec, nxy, float(g["dx"]), float(g["dz"]))
    _write(f"{d}/m.vp", g["vp"])
    _write(f"{d}/m.src", srcA)
    _write(f"{d}/m.rec", recA)
    _write(f"{d}/m.ref", g["Z"])
    inp = _inp2d(d, 160, 600, 12.5, 8.0, len(srnum), len(rec), 4, g["Z"].shape[0])
    r = _run("RT_PFAST2D_FW_NoS", inp)
    assert r.returncode == 0, r.stdout + r.stderr
    Tr = np.fromfile(f"{d}/m_Tr2D.bin").reshape(-1, 3)     # prefix = model path minus ".vp"
    assert Tr.shape[0] == len(rec)
    assert bits_equal(Tr[g["rows"], 0], g["tt"])
    assert bits_equal(Tr[g["rows"], 2], g["tr2"])


def test_rt_pfast2d_fw_shot_gathers_match_oracle(tmp_path):
    from oracle import port
    d = str(tmp_path)
    NX, NY, dx, dz = 40, 90, 10.0, 10.0
    vp = 1600.0 + 20.0 * np.arange(NX)[:, None] + np.zeros((1, NY))
    Z = np.stack([np.full(NY, 250.0), -np.ones(NY), np.zeros(NY)], 1)
    src = np.array([[0, 10], [0, 70]], np.int32)
    rec = np.array([(0, j) for j in range(0, NY, 3)] * 2, np.int32)
    srnum = np.full(2, len(rec) // 2, np.int32)
    nxy = np.tile([-1.0, 0.0], (len(rec), 1))
    srcA, recA = _metres2d(src, srnum, rec, nxy, dx, dz)
    _write(f"{d}/m.vp", vp)
    _write(f"{d}/m.src", srcA)
    _write(f"{d}/m.rec", recA)
    _write(f"{d}/m.ref", Z)
    inp = _inp2d(d, NX, NY, dx, dz, 2, len(rec), 4, NY)
    r = _run("RT_PFAST2D_FW", inp)
    assert r.returncode == 0, r.stdout + r.stderr
    Tr_ref, st = port.forward2d(vp, Z, src, srnum, rec, 1, 500, dx, dz)
    assert bits_equal(np.fromfile(f"{d}/m_Tr2D.bin").reshape(-1, 2), Tr_ref)
    for s in range(2):
        _, TTd, TTu, _, _ = port.rt_fsm2d(vp, Z, src, s, 1, 500, dx, dz)
        assert bits_equal(np.fromfile(f"{d}/m_Src{s}_TTd.2d").reshape(1, NX, NY), TTd)
        assert bits_equal(np.fromfile(f"{d}/m_Src{s}_TTu.2d").reshape(1, NX, NY), TTu)


def _inp3d(d, NX, NY, NZ, dx, dy, dz, nsrc, nrec):
    text = f"""# drop-in test
{d}/m3.vp
{d}/m3.src
{nsrc} 4
{d}/m3.rec
{nrec} 7
{NX} {NY} {NZ} {dx} {dy} {dz}
{d}/out.vp
200 200 10
3 2
"""
    p = os.path.join(d, "case3.inp")
    open(p, "w").write(text)
    return p


def test_t_pfast3d_fw_matches_oracle(tmp_path):
    from oracle import port
    d = str(tmp_path)
    NZ, NX, NY = 10, 14, 40
    dx, dy, dz = 20.0, 20.0, 10.0
    rng = np.random.default_rng(4)
    vp = 1800.0 + 1500.0 * rng.random((NZ, NX, NY))
    src = np.array([[3, 5, 0], [13, 39, 2]], np.int32)                    # (row, col, z)
    r1 = np.array([(i, j, 0) for i in range(0, NX, 3) for j in range(0, NY, 5)], np.int32)
    rec = np.concatenate([r1, r1])
    srnum = np.full(2, len(r1), np.int32)
    srcA = np.stack([(src[:, 0] + 1) * dy, (src[:, 1] + 1) * dx, (src[:, 2] + 1) * dz, srnum.astype(float)], 1)
    recA = np.stack([(rec[:, 0] + 1) * dy, (rec[:, 1] + 1) * dx, (rec[:, 2] + 1) * dz,
                     np.zeros(len(rec)), np.zeros(len(rec)), -np.ones(len(rec)), np.zeros(len(rec))], 1)
    _write(f"{d}/m3.vp", vp)
    _write(f"{d}/m3.src", srcA)
    _write(f"{d}/m3.rec", recA)
    inp = _inp3d(d, NX, NY, NZ, dx, dy, dz, 2, len(rec))
    r = _run("T_PFAST3D_FW", inp)
    assert r.returncode == 0, r.stdout + r.stderr
    want = port.forward3d(vp, src, srnum, rec, 100, dx, dy, dz)
    assert bits_equal(np.fromfile(f"{d}/m3_Tr3D.bin"), want)
    # a source where vp < 400 is rejected, as the reference does (src/T_PFAST3D.cpp:253-256)
    vp[0, 3, 5] = 330.0
    _write(f"{d}/m3.vp", vp)
    r = _run("T_PFAST3D_FW", inp)
    assert r.returncode == 1 and "not in the model volume" in r.stdout


# ------------------------------------------------------------------ inverse drop-ins
def _inp2d_inv(d, NX, NY, dx, dz, nsrc, nrec, rNY, gmNX, nux, nuz, scheme, lsrc):
    text = f"""# inversion drop-in test
{d}/m.vp
{d}/m.src
{nsrc} 3
{d}/m.rec
{nrec} {rNY}
{d}/m.ref
{gmNX} 3
{NX}.000000 {NY}.000000 {dx} {dz}
{d}/final.vp
{nux} {nuz}
{d}/m.wr
{scheme} {lsrc}
"""
    p = os.path.join(d, "inv.inp")
    open(p, "w").write(text)
    return p


def test_rt_pfast2d_inverse_prints_the_reference_trace(tmp_path):
    """RT_PFAST2D on the shipped inversion inputs (metres, 7-column receiver file) for two
    iterations: the residual and line-search lines equal the reference's log, and the files
    of each iteration are written."""
    from helpers import load_inv, load_trace
    g, inv, tr = load_fw(), load_inv(), load_trace()
    d = str(tmp_path)
    src, srnum, rec = g["src"], g["srnum"], g["rec"].astype(np.int32)
    srcA, recA = _metres2d(src, srnum, rec, tr["nxy"], 12.5, 8.0)
    recA = np.concatenate([recA, tr["tt"][:, None], tr["tr"]], 1)
    _write(f"{d}/m.vp", inv["vp"])
    _write(f"{d}/m.src", srcA)
    _write(f"{d}/m.rec", recA)
    _write(f"{d}/m.ref", g["Z"])
    _write(f"{d}/m.wr", np.full((160, 600), 0.5))
    inp = _inp2d_inv(d, 160, 600, 12.5, 8.0, 56, 33600, 7, 1200, 60, 20, 3, 2)
    r = subprocess.run([os.path.join(BIN, "RT_PFAST2D"), inp, "50"], capture_output=True, text=True,
                       env=dict(os.environ, PFAST_MAXITER="2"))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    got = [l for l in r.stdout.splitlines() if l.startswith(("Average Time Residual", "(alpha0,alpha1"))]
    want = [str(s) for s in tr["log_rttag3"]]
    assert got == want[:len(got)] and len(got) == 5
    for k in (1, 2):
        for part in ("RT", "R", "T"):
            for stage in ("bf", "af"):
                assert os.path.getsize(f"{d}/m_{stage}_regu_{part}{k}") == 8 * 96000
        assert os.path.getsize(f"{d}/m_{k}") == 8 * 96000
    assert np.array_equal(np.fromfile(f"{d}/final.vp"), np.fromfile(f"{d}/m_2"))
    assert len(open(f"{d}/m_GlobalErr_TR_T_R.txt").read().splitlines()) == 2
    assert len(open(f"{d}/m_AveRes_TR_T_R.txt").read().splitlines()) == 2


def _case3d_inv():
    from test_gpu_invert import _case3d
    return _case3d()


def _inp3d_inv(d, vpname, NX, NY, NZ, h, nsrc, nrec, lsrc):
    text = f"""# inversion drop-in test
{d}/{vpname}
{d}/m3.src
{nsrc} 4
{d}/m3.rec
{nrec} 7
{NX} {NY} {NZ} {h} {h} {h}
{d}/final3.vp
30 30 20
3 {lsrc}
"""
    p = os.path.join(d, "inv3.inp")
    open(p, "w").write(text)
    return p


def test_t_pfast3d_inverse_and_resume_match_oracle(tmp_path, ctx):
    """T_PFAST3D for one iteration, then a resume of iteration 2 from the files a stopped run
    leaves (<p>.vp1, <p>_bf_regu_1.vp, <p>_bf_regu_2.vp, global_E.tmp, alpha1.tmp): the models
    equal the oracle loop's (with the same resume) to 1e-9."""
    import pfast_gb300 as pg
    import torch
    from oracle import invert as oinv
    bg, src, srnum, rec, nxyz, tobs, (nz, nr, nc), h = _case3d_inv()
    d = str(tmp_path)
    srcA = np.stack([(src[:, 0] + 1) * h, (src[:, 1] + 1) * h, (src[:, 2] + 1) * h, srnum.astype(float)], 1)
    recA = np.concatenate([(rec + 1) * h, nxyz, tobs[:, None]], 1)
    _write(f"{d}/m3.vp", bg)
    _write(f"{d}/m3.src", srcA)
    _write(f"{d}/m3.rec", recA)
    exe = os.path.join(BIN, "T_PFAST3D")
    r = subprocess.run([exe, _inp3d_inv(d, "m3.vp", nr, nc, nz, h, len(src), len(rec), 2), "2"], capture_output=True,
                       text=True, cwd=d, env=dict(os.environ, PFAST_MAXITER="1"))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    loop = oinv.loop3d(bg, src, srnum, rec, nxyz, tobs, h, h, h, 30.0, 30.0, 20.0, lsrc=2, LM=2, nthreads=8)
    loop.step()
    vp1 = np.fromfile(f"{d}/m3.vp1").reshape(nz, nr, nc)
    assert np.allclose(vp1, loop.vp, rtol=1e-9, atol=0)
    # what a run stopped inside iteration 2 leaves: iteration 2's raw gradient and misfit
    sv = pg.Survey3D(ctx, nr, nc, nz, h, h, h, src, srnum, rec, nxyz, tobs)
    g2, E2, _ = sv.eval(torch.from_numpy(vp1).cuda())
    g2 = g2.cpu().numpy()
    sv.close()
    _write(f"{d}/m3_bf_regu_2.vp", g2)
    E1 = float(open(f"{d}/m3_GlobalErr.txt").read().split()[0])
    open(f"{d}/global_E.tmp", "w").write(f"{E1:g}\n{E2:g}\n")
    a1 = float(open(f"{d}/alpha1.tmp").read().split()[0])
    r = subprocess.run([exe, _inp3d_inv(d, "m3.vp1", nr, nc, nz, h, len(src), len(rec), 2), "2"],
                       capture_output=True, text=True, cwd=d, env=dict(os.environ, PFAST_MAXITER="2"))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    assert "Iterating No. 1 resumed" in r.stdout and "Iterating No. 2 started" in r.stdout
    g1 = np.fromfile(f"{d}/m3_bf_regu_1.vp")
    res = oinv.loop3d(vp1, src, srnum, rec, nxyz, tobs, h, h, h, 30.0, 30.0, 20.0, lsrc=2, LM=2, nthreads=8)
    res.resume(1, g1, g2, [float(f"{E1:g}"), float(f"{E2:g}")], a1)
    res.step()
    vp2 = np.fromfile(f"{d}/m3.vp2").reshape(nz, nr, nc)
    assert np.allclose(vp2, res.vp, rtol=1e-9, atol=0)
    assert np.array_equal(np.fromfile(f"{d}/final3.vp").reshape(nz, nr, nc), vp2)
