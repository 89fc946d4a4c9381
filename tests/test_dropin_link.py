"""The drop-in shim links into the reference's own driver: the unchanged
src/eprem.c main() resolves updateEnergeticParticles / updateMhd / moveNodes /
masMoveNodes / rotSunAndSpawnShell, and the wrappers of dataDumpIO and
initEnergeticParticles, to eprem_gb300/host/eprem_dropin.c, which calls the C
ABI.  Needs the
reference source tree (present in the build container only)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _orc  # noqa: E402  (the reference tree's location only)

REF = _orc.reference_root() or ""

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="reference source tree not present")


def test_driver_links_against_dropin():
    lib = os.path.join(ROOT, "eprem_gb300", "libeprem_gpu.so")
    if not os.path.exists(lib):
        from eprem_gb300 import build
        build.build()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "eprem_gb300", "host"), "link",
                           f"REF={REF}"])
    exe = os.path.join(ROOT, "eprem_gb300", "host", "_link", "eprem_gb300")
    syms = subprocess.check_output(["nm", exe], text=True)
    defined = {ln.split()[-1] for ln in syms.splitlines() if " T " in ln}
    for name in ("updateEnergeticParticles", "updateMhd", "moveNodes", "masMoveNodes",
                 "rotSunAndSpawnShell", "dataDumpIO", "initEnergeticParticles", "main"):
        assert name in defined
    # the reference bodies are kept under other names; the driver calls the shim
    for name in ("updateEnergeticParticles_cpu", "updateMhd_cpu", "moveNodes_cpu",
                 "masMoveNodes_cpu", "rotSunAndSpawnShell_cpu", "dataDumpIO_cpu",
                 "initEnergeticParticles_cpu"):
        assert name in defined
    undefined = {ln.split()[-1] for ln in syms.splitlines() if " U " in ln}
    assert {"eprem_gpu_create", "eprem_gpu_update_energetic_particles", "eprem_gpu_ripple_f",
            "eprem_gpu_upload_f_pitched", "eprem_gpu_download_f_pitched",
            "eprem_gpu_update_mhd", "eprem_gpu_move_nodes", "eprem_gpu_mas_init",
            "eprem_gpu_mas_load_slice", "eprem_gpu_mas_select", "eprem_gpu_mas_move_nodes",
            "eprem_gpu_mas_use"} <= undefined
