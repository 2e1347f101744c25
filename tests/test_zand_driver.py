"""The GPU ``zand`` driver run like the reference: a run directory with
``Initial.py``, ``Bias.py`` and ``Arrays/`` in, ``<name>_save/`` out.

Outputs are compared with the fixture recorded from the unmodified reference
run of the same inputs: the time grid and lead currents at 1e-10 (FP64 path),
the complex64 density matrices at 1e-6.
"""
import glob
import os
import re

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _write_run(d, z, saveevery, device_dH=False, usesave=False, t1=None, extra=()):
    from zandpack_gb300.arrays_io import write_arrays
    from zandpack_gb300.workloads import Workload
    p = z["params"]
    keys = ["H_Ortho", "DM_Ortho", "psi_shape", "Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M",
            "diff_GGP_GLP", "diff_GGM_GLM", "xi", "Ixi", "zero_tol"]
    if "S^(-0.5)" in z:
        keys.append("S^(-0.5)")
    write_arrays(os.path.join(d, "run", "Arrays"), {k: z[k] for k in keys})
    w = Workload("gold", {}, p["t0"], p["t1"], p["eps"], p["stepsize"], p["hbar"], p["bias"], p["hubbard_U"],
                 0.025, [])
    with open(os.path.join(d, "Initial.py"), "w") as f:
        f.write("\n".join([
            "from Zandpack.td_constants import hbar",
            "from Zandpack.Loader import load_dictionary",
            "hbar=%r" % p["hbar"], "name='run'", "t0=%r" % p["t0"], "t1=%r" % (t1 or p["t1"]),
            "eps=%r" % p["eps"], "usesave=%r" % usesave, "LoadFromFull=True",
            "checkpoints=[%r]" % (0.5 * p["t1"]), "save_checkpoints=True", "print_timings=False",
            "stepsize=%r" % p["stepsize"], "n_dm_compress=1", "save_PI=True", "saveevery=%d" % saveevery,
            "Arrs=load_dictionary('run/Arrays/')"] + list(extra) + [""]))
    src = w.bias_source()
    if device_dH and p["hubbard_U"] is not None:
        src += "dH_device = {'kind': 'hubbard', 'U': %r}\n" % p["hubbard_U"]
    with open(os.path.join(d, "Bias.py"), "w") as f:
        f.write("from mpi4py import MPI\n" + src)


def _collect(save):
    def steps(pat):
        out = {}
        for f in glob.glob(os.path.join(save, pat)):
            m = re.search(r"(\d+)\.npy$", f)
            out[int(m.group(1))] = np.load(f)
        return [out[k] for k in sorted(out)]
    times = np.concatenate([np.ravel(x) for x in steps("times*.npy")])
    cur = [np.concatenate([np.ravel(x) for x in steps("current_%d_*.npy" % a)]) for a in range(2)]
    dm = np.concatenate(steps("DM[0-9]*.npy"))
    return times, np.array(cur), dm


def test_nozand_driver_matches_reference_run(tmp_path):
    """``nozand`` through the GPU driver against the unmodified reference
    nozand's recorded run: time grid and currents at 1e-10, sigma' (complex64
    DM files) at 1e-6."""
    from zandpack_gb300.zand import ZandRun
    z = load_golden("nz_mini2")
    _write_run(str(tmp_path), z, saveevery=1, device_dH=True)
    cwd = os.getcwd()
    try:
        ZandRun(str(tmp_path), log=lambda *a: None, nonorth=True).run()
    finally:
        os.chdir(cwd)
    times, cur, dm = _collect(str(tmp_path / "run_save"))
    np.testing.assert_allclose(times, z["times"], rtol=0, atol=1e-10)
    assert np.abs(cur - z["currents"]).max() < 1e-10
    assert np.abs(dm[z["sig_traj_idx"] + 1] - z["sig_traj"]).max() < 1e-6


def test_nozand_driver_output_flags(tmp_path):
    """compress_mat, dm_triu_only and dm_occ_only: the DM archives hold the
    plain run's sigma' with the strict lower triangle and the entries where
    |S| <= 1e-6 zeroed (Zandpack/mpi/nozand:547-560)."""
    from zandpack_gb300.arrays_io import flexload
    from zandpack_gb300.zand import ZandRun
    z = load_golden("nz_mini2")
    runs = {}
    for flags in ((), ("compress_mat=True", "dm_triu_only=True", "dm_occ_only=True")):
        d = tmp_path / ("f%d" % len(flags))
        d.mkdir()
        _write_run(str(d), z, saveevery=4, device_dH=True, t1=0.3, extra=flags)
        cwd = os.getcwd()
        try:
            ZandRun(str(d), log=lambda *a: None, nonorth=True).run()
        finally:
            os.chdir(cwd)
        save = str(d / "run_save")
        ext = ".npz" if flags else ".npy"
        files = sorted(glob.glob(os.path.join(save, "DM[0-9]*" + ext)),
                       key=lambda f: int(re.search(r"(\d+)\.np[yz]$", f).group(1)))
        assert files
        runs[len(flags)] = np.concatenate([flexload(f) for f in files])
    Sm05 = np.asarray(z["S^(-0.5)"])[0]
    S05 = np.linalg.inv(Sm05)
    mask = np.abs(S05 @ S05) > 1e-6
    np.testing.assert_array_equal(runs[3], np.triu(runs[0] * mask))


@pytest.mark.parametrize("device_dH", [False, True])
def test_driver_matches_reference_run(tmp_path, device_dH):
    from zandpack_gb300.zand import ZandRun
    z = load_golden("mini2")
    _write_run(str(tmp_path), z, saveevery=1, device_dH=device_dH)
    cwd = os.getcwd()
    try:
        ZandRun(str(tmp_path), log=lambda *a: None).run()
    finally:
        os.chdir(cwd)
    times, cur, dm = _collect(str(tmp_path / "run_save"))
    np.testing.assert_allclose(times, z["times"], rtol=0, atol=1e-10)
    assert np.abs(cur - z["currents"]).max() < 1e-10
    # DM files hold every accepted sigma (complex64)
    assert np.abs(dm[z["sig_traj_idx"] + 1] - z["sig_traj"]).max() < 1e-6
    assert os.path.exists(tmp_path / "run_save" / "last_psi.npy")
    # the reference's readers (mpi_tools names) read the same run back
    from zandpack_gb300.mpi_tools import combine_currents, combine_dm
    T, C = combine_currents([str(tmp_path / "run_save")])
    np.testing.assert_allclose(T, z["times"][:-1], rtol=0, atol=1e-10)
    assert np.abs(np.hstack([c[:, 0][:, None] for c in C]).T - z["currents"]).max() < 1e-10
    Td, DMr = combine_dm([str(tmp_path / "run_save")])
    np.testing.assert_allclose(Td, z["times"], rtol=0, atol=1e-10)
    np.testing.assert_array_equal(DMr, dm)


def test_driver_restart_from_checkpoint(tmp_path):
    """A run stopped at its checkpoint and resumed (usesave, LoadFromFull)
    lands on the same final sigma as the uninterrupted run."""
    from zandpack_gb300.zand import ZandRun
    z = load_golden("mini2")
    p = z["params"]
    _write_run(str(tmp_path), z, saveevery=1000)
    cwd = os.getcwd()
    try:
        full = ZandRun(str(tmp_path), log=lambda *a: None).run()
        sig_full = full.prop.traj.get_y()[0]
        t_full = full.t_end
        # resume from the checkpoint written at t > t1/2
        _write_run(str(tmp_path), z, saveevery=1000, usesave=True)
        part = ZandRun(str(tmp_path), log=lambda *a: None).run()
        sig_part = part.prop.traj.get_y()[0]
    finally:
        os.chdir(cwd)
    assert abs(part.t_end - t_full) < 1e-12
    assert np.abs(sig_part - sig_full).max() < 1e-12
