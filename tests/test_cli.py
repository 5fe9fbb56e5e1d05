"""The ppgpu command-line driver: a reference input file run on the GPU engine writes the reference's output
files. The checkerboard trajectory differs from the reference's sequential one, so the step-0 lines (the
uploaded configuration's exact energy, density and box) must equal the reference's own outputs
(tests/golden/traj_*), and every other line must have the reference's format and cadence. Input errors are
checked on the CPU (they stop the driver before it touches a GPU)."""
import gzip
import os
import shutil
import subprocess
import tempfile

import pytest

from patchyparticles_gb300 import build
from tests import helpers

CLI = build.CLI


def _prepare(name, edit=None):
    src = helpers.golden_path("traj_" + name)
    work = tempfile.mkdtemp(prefix="ppcli_")
    os.makedirs(os.path.join(work, "confs"))
    text = open(os.path.join(src, "input")).read()
    if edit:
        text = edit(text)
    open(os.path.join(work, "input"), "w").write(text)
    if "Umbrella_sampling_folder" in text:
        os.makedirs(os.path.join(work, "sus"))
    conf = [l.split("=")[1].strip() for l in text.splitlines() if l.startswith("Initial_conditions_file")][0]
    helpers.unpack_golden(conf, work)
    return src, work


def _lines(path):
    return helpers.normalise_nan(open(path).read()).splitlines()


@pytest.mark.gpu
@pytest.mark.parametrize("name,files", [("small_nvt", ("energy.dat", "acceptance.dat")),
                                        ("small_npt", ("energy.dat", "acceptance.dat", "density.dat")),
                                        ("small_lx", ("energy.dat", "acceptance.dat", "boxshape.dat")),
                                        ("small_gc", ("energy.dat", "acceptance.dat", "density.dat")),
                                        ("small_sus", ("energy.dat", "acceptance.dat", "density.dat")),
                                        ("small_avb", ("energy.dat", "acceptance.dat")),
                                        ("small_avb_npt", ("energy.dat", "acceptance.dat", "density.dat")),
                                        ("small_vmmc", ("energy.dat", "acceptance.dat")),
                                        ("small_vmmc_npt", ("energy.dat", "acceptance.dat", "density.dat"))])
def test_driver_writes_the_reference_outputs(built, name, files):
    src, work = _prepare(name)
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    ref_out = open(os.path.join(src, "stdout.txt")).read().splitlines()
    out = p.stdout.splitlines()
    assert len(out) == len(ref_out) and out[0] == ref_out[0]
    assert out[-1].split()[0] == ref_out[-1].split()[0]  # the final step
    for fn in files:
        mine, ref = _lines(os.path.join(work, fn)), _lines(os.path.join(src, fn))
        assert len(mine) == len(ref), fn
        assert mine[0] == ref[0], fn  # step 0: the uploaded configuration
        for a, b in zip(mine, ref):
            assert a.split()[0] == b.split()[0] and len(a.split()) == len(b.split()), fn
    last = open(os.path.join(work, "last.rrr")).read().splitlines()
    ref_last = gzip.open(os.path.join(src, "last.rrr.gz"), "rt").read().splitlines()
    if os.path.exists(os.path.join(src, "density.dat")) and "Activity" in open(os.path.join(src, "input")).read():
        # GC / SUS: the particle count of the last configuration is the run's own
        assert last[0].split()[0] == ref_last[0].split()[0] and len(last) == 1 + 3 * int(last[0].split()[1])
    else:
        assert len(last) == len(ref_last) and last[0].split()[:2] == ref_last[0].split()[:2]
    saves = sorted(os.listdir(os.path.join(work, "confs")))
    assert saves and all(f.startswith("conf_") and f.endswith(".rrr") for f in saves)
    if os.path.isdir(os.path.join(src, "sus")):  # one histogram file per print after step 0 (main.c:89)
        assert sorted(os.listdir(os.path.join(work, "sus"))) == sorted(os.listdir(os.path.join(src, "sus")))
        for fn in os.listdir(os.path.join(work, "sus")):
            for line in open(os.path.join(work, "sus", fn)):
                n, c = map(int, line.split())
                assert 295 <= n <= 305 and c > 0
    shutil.rmtree(work)


@pytest.mark.gpu
def test_driver_writes_bond_files(built):
    """Print_bonds: bonds_<step>.dat at every print; at step 0 the partner sets equal the reference's own
    per-particle probe of the same configuration (output_print_bonds, output.c:213-268)."""
    src, work = _prepare("small_nvt", lambda t: t + "Print_bonds = 1\nBonds_folder = bonds\n")
    os.makedirs(os.path.join(work, "bonds"))
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    files = sorted(os.listdir(os.path.join(work, "bonds")))
    assert "bonds_0.dat" in files and len(files) == len(open(os.path.join(src, "energy.dat")).read().splitlines())
    lines = open(os.path.join(work, "bonds", "bonds_0.dat")).read().splitlines()
    N, _, _, _, _, nb, _, bonded = helpers.parse_probe("small")
    assert int(lines[0]) == N and len(lines) == 1 + 2 * N
    for i in range(N):
        idx, n = map(int, lines[1 + 2 * i].split())
        partners = [int(v) for v in lines[2 + 2 * i].split()]
        assert idx == i and n == nb[i] == len(partners) and sorted(partners) == sorted(bonded[i])
    shutil.rmtree(work)


@pytest.mark.gpu
def test_driver_refuses_an_overlapping_configuration(built):
    src, work = _prepare("small_nvt", lambda t: t.replace("generator_300_0.3_4242.rrr", "adversarial.rrr"))
    helpers.unpack_golden("adversarial.rrr", work)
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=300)
    assert p.returncode == 1 and "Initial configuration contains an overlap, aborting" in p.stderr
    shutil.rmtree(work)


def test_driver_reports_a_missing_mandatory_key(built):
    src, work = _prepare("small_nvt", lambda t: "\n".join(l for l in t.splitlines() if not l.startswith("Temperature")))
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=60)
    assert p.returncode == 255 and "Mandatory key 'Temperature' not found" in p.stderr
    shutil.rmtree(work)


def test_driver_rejects_other_dynamics(built):
    src, work = _prepare("small_nvt", lambda t: t.replace("Dynamics = 0", "Dynamics = 3"))
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=60)
    assert p.returncode == 1 and "Dynamics = 3" in p.stderr
    shutil.rmtree(work)


def test_driver_needs_the_vmmc_keys(built):
    src, work = _prepare("small_nvt", lambda t: t.replace("Dynamics = 0", "Dynamics = 1"))
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=60)
    assert p.returncode == 255 and "Mandatory key 'vmmc_max_move' not found" in p.stderr  # vmmc.c:22
    shutil.rmtree(work)


@pytest.mark.parametrize("edit,code,msg", [
    (lambda t: t.replace("Ensemble = 0", "Ensemble = 2"), 1, "Ensemble = 2"),
    (lambda t: t.replace("generator_300_0.3_4242.rrr", "missing.rrr"), 1, "missing.rrr"),
    (lambda t: t + "Print_bonds = 1\n", 255, "Mandatory key 'Bonds_folder' not found"),
    (lambda t: t + "Print_bonds = 1\nBonds_folder = nowhere\n", 1, "Cannot create files in directory 'nowhere'"),
])
def test_driver_input_errors(built, edit, code, msg):
    src, work = _prepare("small_nvt")
    path = os.path.join(work, "input")
    text = edit(open(path).read())
    open(path, "w").write(text)
    p = subprocess.run([CLI, "input"], cwd=work, capture_output=True, text=True, timeout=60)
    assert p.returncode == code and msg in p.stderr, p.stderr
    shutil.rmtree(work)


@pytest.mark.gpu
def test_sigterm_stops_between_output_blocks_and_writes_the_last_configuration(built):
    """main.c:15-39: SIGTERM sets the stop flag; the loop ends after the current block of sweeps, the final
    configuration and line are written and the exit status is 0."""
    import signal

    src, work = _prepare("small_nvt", lambda t: t.replace("Steps = 200", "Steps = 1000000000").replace("Print_every = 20", "Print_every = 200")
                         .replace("Save_every = 40", "Save_every = 1000000"))
    p = subprocess.Popen([CLI, "input"], cwd=work, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    lines = []
    try:
        while len(lines) < 3:  # in the main loop: the handler is installed and several blocks have run
            line = p.stdout.readline()
            assert line, p.stderr.read()
            lines.append(line)
        p.send_signal(signal.SIGTERM)
        out, err = p.communicate(timeout=120)
    finally:
        if p.poll() is None:
            p.kill()
    assert p.returncode == 0, err
    lines += out.splitlines()
    final = int(lines[-1].split()[0])
    assert 400 <= final < 1000000000 and final % 200 == 0
    last = open(os.path.join(work, "last.rrr")).read().splitlines()
    assert int(last[0].split()[0]) == final and int(last[0].split()[1]) == 300 and len(last) == 1 + 3 * 300
    shutil.rmtree(work)
