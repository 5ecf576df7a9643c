"""Generates the golden fixtures in tests/golden/ from the FilterBSE reference
tree (run here, where the reference is mounted; the fixtures are committed so
the tests never read the reference at run time).

Fixtures (all data outputs or inputs of the reference's own example runs):
  zn_2048.txt            Leja/Ashkenazy nodes written by gen_newton_coeff
                         (coeff.c:66-71) for nCheby = 2048 (filter.zip,
                         filter/2.2nm_CdSe/zn.dat), "%ld %lg" format
  seed_2.2nm_CdSe.txt    seed sequence of init_filter_states (init.c:729-741),
                         one state = 57*52*45 real draws (filter.zip seed.dat)
  ksqr_57x52x45.txt      every 61st line (plus the first 200) of ksqr.dat
                         written by build_grid_ksqr (init.c:338-351) for
                         dx = 0.8, KEmax = 10 (filter.zip ksqr.dat)
  cdse22/                2.2 nm CdSe example: conf.par, the II-VI potential
                         tables, eval.dat of the reference run, and every 37th
                         value of its localPot.cube (build_local_pot output,
                         "%.5g") with the grid header
  cspbi3/                1x1x1 CsPbI3 spinor SO+NL example: input.par,
                         conf.par, pot*.par, SO_*.par and reference eval.dat;
                         its BSE run (bse_cplx/EXAMPLES/1x1x1_CsPbI3/bse):
                         bse_input.par and the reference's exciton.dat,
                         OS.dat, OS0.dat, M0.dat, M.dat, rs0.dat, rs.dat and
                         the calcSpinAngStat files lsqr.dat, ls.dat,
                         spins.dat, orbital.dat, couple.dat, qp_spins.dat
  inp/                   the In and P local-potential tables shipped with the
                         In13P16 example (filter.zip, filter/In13_P16/potIn.par,
                         potP.par), for the InP dots of the multi-dot workload
"""
import os
import shutil
import zipfile

REF = "/root/reference"
OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    z = zipfile.ZipFile(os.path.join(REF, "filter.zip"))
    with open(os.path.join(OUT, "zn_2048.txt"), "wb") as f:
        f.write(z.read("filter/2.2nm_CdSe/zn.dat"))
    with open(os.path.join(OUT, "seed_2.2nm_CdSe.txt"), "wb") as f:
        f.write(z.read("filter/2.2nm_CdSe/seed.dat"))
    lines = z.read("filter/2.2nm_CdSe/ksqr.dat").decode().splitlines()
    keep = [l for i, l in enumerate(lines) if i < 200 or i % 61 == 0]
    with open(os.path.join(OUT, "ksqr_57x52x45.txt"), "w") as f:
        f.write("# nx ny nz dx KEmax: 57 52 45 0.8 10\n")
        f.write("\n".join(keep) + "\n")

    ex = os.path.join(REF, "filter_mpi", "EXAMPLES")
    d = os.path.join(OUT, "cdse22")
    os.makedirs(d, exist_ok=True)
    shutil.copy(os.path.join(ex, "2.2nm_CdSe", "conf.par"), d)
    shutil.copy(os.path.join(ex, "2.2nm_CdSe", "filter", "input.par"), d)
    shutil.copy(os.path.join(ex, "2.2nm_CdSe", "filter", "eval.dat"), d)
    for a in ("Cd", "Se", "P1", "P2"):
        shutil.copy(os.path.join(REF, "pots", "pots_II_VI", f"pot{a}.par"), d)
    cube = open(os.path.join(ex, "2.2nm_CdSe", "filter", "localPot.cube")).read().splitlines()
    hdr = cube[:6]
    natoms = int(hdr[2].split()[0])
    vals = " ".join(cube[6 + natoms:]).split()
    with open(os.path.join(d, "localPot_sample.txt"), "w") as f:
        f.write("# cube header (xmin ymin zmin; n d per axis), then 'cube_index value' for every 37th value\n")
        f.write("# cube order: x outer, y middle, z inner\n")
        for h in hdr[2:6]:
            f.write("# " + h + "\n")
        for i in range(0, len(vals), 37):
            f.write(f"{i} {vals[i]}\n")

    d = os.path.join(OUT, "cspbi3")
    os.makedirs(d, exist_ok=True)
    src = os.path.join(ex, "1x1x1_CsPbI3", "filter")
    for fn in ("input.par", "conf.par", "potCs.par", "potI.par", "potPb.par", "SO_Cs.par", "SO_I.par", "SO_Pb.par"):
        shutil.copy(os.path.join(src, fn), d)
    shutil.copy(os.path.join(src, "reference_output", "eval.dat"), d)
    di = os.path.join(OUT, "inp")
    os.makedirs(di, exist_ok=True)
    for a in ("In", "P"):
        with open(os.path.join(di, f"pot{a}.par"), "wb") as f:
            f.write(z.read(f"filter/In13_P16/pot{a}.par"))
    bse = os.path.join(REF, "bse_cplx", "EXAMPLES", "1x1x1_CsPbI3", "bse")
    shutil.copy(os.path.join(bse, "input.par"), os.path.join(d, "bse_input.par"))
    for fn in ("exciton.dat", "OS.dat", "OS0.dat", "M0.dat", "M.dat", "rs0.dat", "rs.dat", "lsqr.dat", "ls.dat",
               "spins.dat", "orbital.dat", "couple.dat", "qp_spins.dat"):
        shutil.copy(os.path.join(bse, "reference_output", fn), d)


if __name__ == "__main__":
    main()
