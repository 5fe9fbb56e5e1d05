"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Run from the repository root in a container where the reference sources are present
(python tests/golden/make_golden.py [reference_dir [output_dir]]); it builds oracle/_ref with
oracle/Makefile and runs the reference's own programs. The fixtures go to tests/golden/ unless an output
directory is given (tests/test_golden_regen.py regenerates them into a scratch directory and compares):

  generator_<N>_<rho>_<seed>.rrr.gz   reference generator seeded with srand48(seed) (oracle/ref_generator_seeded.c)
  probe_<name>.txt.gz                 ref_probe: per-particle MC_energy, overlap flag, bond/overlap partners
  traj_<name>/                        reference main loop outputs (stdout, energy/acceptance/density/boxshape, last.rrr)
  adversarial.rrr.gz                  near-threshold pair configuration (tests/golden/adversarial.py)

The reference is compiled with -O2 -ffp-contract=off (oracle/Makefile); nothing here is used at run time
on a machine without the reference: tests read only the committed outputs.
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle.pyoracle import reference_dir  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else reference_dir()
if REF is None:
    sys.exit("reference sources not found: pass their directory or set PP_REFERENCE_DIR")
OUT = sys.argv[2] if len(sys.argv) > 2 else HERE
REFOUT = os.path.join(ROOT, "oracle", "_ref")

# synthetic configurations: (name, N, density, seed) -- shapes of the benchmark configurations at sizes the
# CPU reference handles in seconds
GENERATED = [
    ("c1", 1000, 0.1, 1001),
    ("c2", 4000, 0.5, 1002),
    ("c3", 2000, 0.6, 1003),
    ("c5", 4000, 0.3, 1005),
    ("small", 300, 0.3, 4242),
]

TRAJ_INPUT = """Dynamics = {dynamics}
Ensemble = {ensemble}
Seed = {seed}
Temperature = {T}
Disp_max = 0.05
Theta_max = 0.1
Steps = {steps}
Print_every = {print_every}
Save_every = {save_every}
Configuration_folder = confs
Initial_conditions_file = {conf}
KF_delta = 0.12
KF_cosmax = 0.92
{extra}"""

TRAJ = [
    # name, conf, ensemble, T, steps, print_every, seed, extra
    ("fcc_nvt", "fcc.rrr", 0, 0.12, 300, 50, 12345, ""),
    ("bcc_npt", "bcc.rrr", 5, 0.12, 400, 50, 12345, "P = 0.05\nrescale_factor_max = 0.01\n"),
    ("small_nvt", "generator_300_0.3_4242.rrr", 0, 0.11, 200, 20, 7, ""),
    ("small_npt", "generator_300_0.3_4242.rrr", 5, 0.11, 300, 30, 9, "P = 0.05\nrescale_factor_max = 0.01\n"),
    # the box-shape move of NVT (MC.c:515-585): Lx changes, Ly = Lz follow at constant volume
    ("small_lx", "generator_300_0.3_4242.rrr", 0, 0.11, 400, 40, 11, "Lx_move = 1\nLx_change_max = 0.5\nLyz_min = 8.0\nLyz_max = 12.0\n"),
    # grand canonical insertions and removals (MC.c:31-43, 342-448) and successive umbrella sampling in an
    # N window (MC.c:45-58, with its histogram files, output.c:343-356)
    ("small_gc", "generator_300_0.3_4242.rrr", 1, 0.12, 300, 30, 13, "Activity = 0.1\nGC_N_max = 600\n"),
    ("small_sus", "generator_300_0.3_4242.rrr", 3, 0.12, 300, 30, 17,
     "Activity = 0.1\nUmbrella_sampling_min = 295\nUmbrella_sampling_max = 305\nUmbrella_sampling_folder = sus\n"),
    # aggregation-volume-bias moves mixed with roto-translations (Dynamics = 2, avb.c:77-186), NVT with the
    # default avb_p and NPT with avb_p = 0.3
    ("small_avb", "generator_300_0.3_4242.rrr", 0, 0.11, 300, 30, 21, "", 2),
    ("small_avb_npt", "generator_300_0.3_4242.rrr", 5, 0.11, 300, 30, 23, "P = 0.05\nrescale_factor_max = 0.01\navb_p = 0.3\n", 2),
    # virtual-move cluster moves (Dynamics = 1, vmmc.c:258-483), NVT and NPT
    ("small_vmmc", "generator_300_0.3_4242.rrr", 0, 0.11, 300, 30, 25, "vmmc_max_move = 0.5\nvmmc_max_cluster = 20\n", 1),
    ("small_vmmc_npt", "generator_300_0.3_4242.rrr", 5, 0.11, 300, 30, 27, "P = 0.05\nrescale_factor_max = 0.01\nvmmc_max_move = 0.5\nvmmc_max_cluster = 10\n", 1),
]

PROBE_INPUT = """Dynamics = 0
Ensemble = 0
Seed = 1
Temperature = 0.12
Disp_max = 0.05
Theta_max = 0.1
Initial_conditions_file = {conf}
KF_delta = 0.12
KF_cosmax = 0.92
"""


def gz_write(path, data):
    """gzip with a zero timestamp, so that regenerating a fixture reproduces its bytes"""
    with open(path, "wb") as raw, gzip.GzipFile(filename="", mode="wb", compresslevel=9, fileobj=raw, mtime=0) as f:
        f.write(data)


def main():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + REF])
    import adversarial

    work = tempfile.mkdtemp()
    # shipped reference fixtures
    for name in ("fcc.rrr", "bcc.rrr"):
        shutil.copy(os.path.join(REF, name), os.path.join(work, name))
        gz_write(os.path.join(OUT, name + ".gz"), open(os.path.join(REF, name), "rb").read())
    # generated configurations
    for name, N, rho, seed in GENERATED:
        subprocess.check_call([os.path.join(REFOUT, "generator_seeded"), str(N), str(rho), str(seed)], cwd=work, stderr=subprocess.DEVNULL)
        fn = "generator_%d_%s_%d.rrr" % (N, rho, seed)
        os.rename(os.path.join(work, "generated.rrr"), os.path.join(work, fn))
        if N <= 1000:
            gz_write(os.path.join(OUT, fn + ".gz"), open(os.path.join(work, fn), "rb").read())
    # adversarial pairs
    r, R, box = adversarial.build(n_pairs=1500)
    adversarial.write_rrr17(os.path.join(work, "adversarial.rrr"), r, R, box)
    gz_write(os.path.join(OUT, "adversarial.rrr.gz"), open(os.path.join(work, "adversarial.rrr"), "rb").read())
    # per-particle probes
    probes = [("fcc", "fcc.rrr"), ("bcc", "bcc.rrr"), ("adversarial", "adversarial.rrr")]
    probes += [(name, "generator_%d_%s_%d.rrr" % (N, rho, seed)) for name, N, rho, seed in GENERATED]
    for name, conf in probes:
        inp = os.path.join(work, "probe_input")
        open(inp, "w").write(PROBE_INPUT.format(conf=conf))
        out = subprocess.check_output([os.path.join(REFOUT, "ref_probe"), inp], cwd=work, stderr=subprocess.DEVNULL)
        gz_write(os.path.join(OUT, "probe_%s.txt.gz" % name), out)
    # trajectories of the reference main loop
    for entry in TRAJ:
        name, conf, ens, T, steps, pe, seed, extra = entry[:8]
        dyn = entry[8] if len(entry) > 8 else 0
        d = os.path.join(work, name)
        os.makedirs(os.path.join(d, "confs"))
        if "Umbrella_sampling_folder" in extra:
            os.makedirs(os.path.join(d, "sus"))
        shutil.copy(os.path.join(work, conf), os.path.join(d, conf))
        open(os.path.join(d, "input"), "w").write(TRAJ_INPUT.format(dynamics=dyn, ensemble=ens, seed=seed, T=T, steps=steps, print_every=pe, save_every=pe * 2, conf=conf, extra=extra))
        out = subprocess.check_output([os.path.join(REFOUT, "PatchyParticles"), "input"], cwd=d, stderr=subprocess.DEVNULL)
        dst = os.path.join(OUT, "traj_" + name)
        os.makedirs(dst, exist_ok=True)
        open(os.path.join(dst, "input"), "w").write(TRAJ_INPUT.format(dynamics=dyn, ensemble=ens, seed=seed, T=T, steps=steps, print_every=pe, save_every=pe * 2, conf=conf, extra=extra))
        open(os.path.join(dst, "stdout.txt"), "wb").write(out)
        for fn in ("energy.dat", "acceptance.dat", "density.dat", "boxshape.dat"):
            if os.path.exists(os.path.join(d, fn)):
                shutil.copy(os.path.join(d, fn), os.path.join(dst, fn))
        gz_write(os.path.join(dst, "last.rrr.gz"), open(os.path.join(d, "last.rrr"), "rb").read())
        if os.path.isdir(os.path.join(d, "sus")):
            os.makedirs(os.path.join(dst, "sus"), exist_ok=True)
            for fn in sorted(os.listdir(os.path.join(d, "sus"))):
                shutil.copy(os.path.join(d, "sus", fn), os.path.join(dst, "sus", fn))
    shutil.rmtree(work)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
