"""Generate the layout view of the reference's data structures that the
reference-signature drop-ins (refshim/mdz_refshim.c) are compiled against
where the reference's own header is not available (the GPU host), and the
same layout as a Python table for the tests that build such structures.

    python mdoodz6.0_gb300/refshim/make_layout.py [REF_SOURCE_DIR] [--check]

It compiles a small program against the reference's SOURCE/header_MDOODZ.h
(with the stand-in SuiteSparse headers of oracle/ref_stubs), which prints the
size of each structure and the offset of each member the drop-ins read or
write.  From these it writes

    include/mdoodz_ref_types.h     each structure as those members at their
                                   offsets, padded in between to the
                                   reference's size (LP64: x86-64 and AArch64
                                   Linux lay these structures out alike)
    refshim/ref_layout.py          {struct: (size, {member: (offset, ctype)})}

--check regenerates both in memory and fails if the committed files differ.
Only the members listed below are described; every other byte is padding.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HEADER_OUT = os.path.join(ROOT, "include", "mdoodz_ref_types.h")
PY_OUT = os.path.join(HERE, "ref_layout.py")
STUBS = os.path.join(ROOT, "oracle", "ref_stubs")

D, I, DP, IP, CP, DPP = "double", "int", "double *", "int *", "char *", "double **"

# the members the drop-ins use, by structure (C type, name)
MEMBERS = {
    "scale": [(D, n) for n in ("eta", "L", "V", "T", "t", "a", "E", "S", "m", "rho", "F", "J", "W", "Cv", "rhoE",
                               "k")],
    "surface": [(DP, n) for n in ("a", "b", "height", "vx", "vz", "a0", "b0", "height0")] + [(IP, "VertInd")],
    "BC": [(CP, "type"), (DP, "val")],
    "BCT": [(CP, "type")],
    "SparseMat": [(DP, "A"), (DP, "x"), (DP, "b"), (DP, "F"), (DP, "d"), (DP, "bbc"), (IP, "Ic"), (IP, "J"),
                  (I, "neq"), (IP, "eqn_u"), (IP, "eqn_v"), (IP, "eqn_p"), (I, "nnz"), (I, "neq_mom"),
                  (I, "neq_cont")],
    "markers": [(I, "Nb_part"), (I, "Nb_part_max"), (I, "min_part_cell")]
               + [(DP, n) for n in ("x", "z", "Vx", "Vz", "P", "sxxd", "szzd", "sxz", "T", "strain", "strain_pl")]
               + [(IP, "phase")],
    "Nparams": [(I, "nit"), (I, "nit_max"), (I, "stagnated"), (D, "abs_tol_u"), (D, "rel_tol_u"), (D, "abs_tol_p"),
                (D, "rel_tol_p"), (D, "resx"), (D, "resz"), (D, "resp"), (D, "resx0"), (D, "resz0"), (D, "resp0"),
                (I, "Picard2Newton"), (I, "nit_Pic_max"), (D, "Pic2NewtCond")],
    "params": [(D, n) for n in ("xmin", "zmin", "xmax", "zmax", "dx", "dz", "dt", "gx", "gz", "mineta", "maxeta",
                                "line_search_min")]
              + [(I, n) for n in ("Nx", "Nz", "step", "Newton", "eta_avg", "itp_stencil", "isperiodic_x",
                                  "iselastic", "free_surf", "line_search", "subgrid_diff", "Nb_phases",
                                  "StressRotation", "StressUpdate", "DirectNeighbour", "Plith_trick", "aniso",
                                  "loc_iter", "lsolver", "diag_scaling")]
              + [(D, "compressible"), (D, "rel_tol_KSP")],
    "mat_prop": [(I, "Nb_phases"), (D, "R")]
                + [(D + "[20]", n) for n in ("eta0", "rho", "mu", "C", "phi", "psi", "Slim", "alp", "bet",
                                            "Qpwl", "Vpwl", "npwl", "mpwl", "Apwl", "apwl", "fpwl", "rpwl", "Fpwl",
                                            "pref_pwl", "Qlin", "Vlin", "nlin", "mlin", "Alin", "alin", "flin",
                                            "rlin", "Flin", "gs_ref", "C_end", "phi_end", "psi_end", "pls_start",
                                            "pls_end", "eta_vp", "n_vp", "Qexp", "Sexp", "Eexp", "Gexp", "nexp",
                                            "Qgbs", "Vgbs", "ngbs", "mgbs", "Agbs", "agbs", "fgbs", "rgbs", "Fgbs")]
                + [(I + "[20]", n) for n in ("gs", "cstv", "pwlv", "linv", "expv", "gbsv", "phi_soft", "psi_soft",
                                            "coh_soft", "is_tensile", "reac_soft", "phase_mix")],
    "grid": [(I, "Nx"), (I, "Nz"), (D, "dx"), (D, "dz")]
            + [(DP, n) for n in (
                "roger_x", "roger_z", "div_u", "div_u_s", "div_u_el", "div_u_pl", "div_u_r", "u_in", "v_in", "p_in",
                "p_corr", "sxxd", "szzd", "sxz", "exxd", "ezzd", "exz", "VE_s", "VE_n", "sxxd0", "szzd0", "sxz0",
                "mu_s", "mu_n", "eta_phys_n", "eta_phys_s",
                "xg_coord", "zg_coord", "xc_coord", "zc_coord", "xvz_coord", "zvx_coord", "eta_s", "eta_n", "rho_s",
                "rho_n", "X_s", "X_n", "X0_s", "X0_n", "p0_n", "p0_s", "OverS_n", "OverS_s", "strain_n", "strain_s",
                "ru", "rv", "rp", "rhs_p", "gx", "gz", "bet_n", "bet_s", "p_lith", "p_lith0", "dp",
                "sxxd0_s", "szzd0_s", "sxz0_n", "exxd_s", "ezzd_s", "exz_n", "sxz_n", "T", "d_n", "d0_n", "phi_n",
                "phi0_n", "eII_el", "eII_pl", "eII_pwl", "eII_exp", "eII_lin", "eII_gbs", "eII_cst", "exx_el",
                "ezz_el", "exz_el", "exx_diss", "ezz_diss", "exz_diss", "D11_n", "D12_n", "D13_n", "D14_n", "D21_n",
                "D22_n", "D23_n", "D24_n", "D31_s", "D32_s", "D33_s", "D34_s", "detadexx_n", "detadezz_n",
                "detadgxz_n", "detadp_n", "ddivpdexx_n", "ddivpdezz_n", "ddivpdgxz_n", "ddivpdp_n", "detadexx_s",
                "detadezz_s", "detadgxz_s", "detadp_s", "phi0_s", "d0_s", "T_s", "P_s", "dil_n", "dil_s", "fric_n",
                "fric_s", "C_n", "C_s", "Wdiss", "Wel", "Wtot")]
            + [(IP, "nb_part_cell"), (IP, "nb_part_vert"), ("BC", "BCu"), ("BC", "BCv"), ("BC", "BCp"),
               ("BCT", "BCg"), ("BCT", "BCt"), (DPP, "phase_perc_n"), (DPP, "phase_perc_s")],
}
ORDER = ["scale", "surface", "BC", "BCT", "SparseMat", "markers", "Nparams", "params", "mat_prop", "grid"]
TAGS = {"scale": "_scale", "surface": "_surface", "BC": "_BC", "BCT": "_BCT", "SparseMat": "_SparseMat",
        "markers": "_p_markers",
        "Nparams": "_n_params", "params": "_params", "mat_prop": "_mat_prop", "grid": "_grid"}


def measure(src_dir):
    prog = ["#include <stdio.h>", "#include <stddef.h>", '#include "header_MDOODZ.h"', "int main(void) {"]
    for s in ORDER:
        prog.append('    printf("%s size %%zu\\n", sizeof(%s));' % (s, s))
        for _, m in MEMBERS[s]:
            prog.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (s, m, s, m))
    prog += ["    return 0;", "}"]
    with tempfile.TemporaryDirectory() as td:
        c, exe = os.path.join(td, "layout.c"), os.path.join(td, "layout")
        with open(c, "w") as fh:
            fh.write("\n".join(prog) + "\n")
        subprocess.run(["gcc", "-std=gnu99", "-w", "-I" + STUBS, "-I" + src_dir, c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    sizes, offs = {}, {}
    for line in out.splitlines():
        s, m, v = line.split()
        if m == "size":
            sizes[s] = int(v)
        else:
            offs[(s, m)] = int(v)
    return sizes, offs


def _decl(ctype, name):
    if ctype.endswith("[20]"):
        return "%s %s[20];" % (ctype[:-4], name)
    if ctype in ("BC", "BCT"):
        return "%s %s;" % (ctype, name)
    if ctype.endswith("*"):
        return "%s%s;" % (ctype, name)
    return "%s %s;" % (ctype, name)


def _csize(ctype, sizes):
    base = ctype.replace("[20]", "")
    n = sizes[base] if base in sizes else {"double": 8, "int": 4}.get(base, 8)
    return n * (20 if ctype.endswith("[20]") else 1)


def render(sizes, offs):
    h = ["/*",
         " * mdoodz_ref_types.h -- layout view of the reference's data structures",
         " * (SOURCE/header_MDOODZ.h: scale, surface, BC, SparseMat, markers, Nparams,",
         " * params, mat_prop, grid) for the reference-signature drop-ins of",
         " * refshim/mdz_refshim.c where the reference's header is not at hand.",
         " *",
         " * GENERATED by mdoodz6.0_gb300/refshim/make_layout.py from the reference's",
         " * header: each structure keeps only the members the drop-ins read or write,",
         " * at the reference's byte offsets (LP64), with padding in between and the",
         " * reference's total size, so that pointers to (and copies of) the caller's",
         " * structures are read correctly.  Do not edit; regenerate.",
         " */",
         "#ifndef MDOODZ_REF_TYPES_H",
         "#define MDOODZ_REF_TYPES_H",
         "#include <stddef.h>",
         "",
         "#define DoodzFP double",
         "",
         "/* the direct solver's state (CHOLMOD): opaque, the drop-ins never read it */",
         "typedef struct _DirectSolver DirectSolver;",
         ""]
    for s in ORDER:
        mem = sorted(MEMBERS[s], key=lambda cm: offs[(s, cm[1])])
        h.append("typedef struct %s %s;" % (TAGS[s], s))
        h.append("struct %s {" % TAGS[s])
        pos, npad = 0, 0
        for ctype, name in mem:
            off = offs[(s, name)]
            if off > pos:
                h.append("    char mdz_pad%d[%d];" % (npad, off - pos))
                npad += 1
            h.append("    " + _decl(ctype, name))
            pos = off + _csize(ctype, sizes)
        if sizes[s] > pos:
            h.append("    char mdz_pad%d[%d];" % (npad, sizes[s] - pos))
        h.append("};")
        h.append("")
    h.append("/* the layout the drop-ins were compiled for */")
    for s in ORDER:
        h.append("_Static_assert(sizeof(%s) == %d, \"%s size\");" % (s, sizes[s], s))
        for _, name in MEMBERS[s]:
            h.append("_Static_assert(offsetof(%s, %s) == %d, \"%s.%s\");" % (s, name, offs[(s, name)], s, name))
    h += ["", "#endif"]
    py = ['"""Layout of the reference\'s structures (struct -> (size, {member: (offset, C type)})),',
          'generated by refshim/make_layout.py together with include/mdoodz_ref_types.h."""', "", "LAYOUT = {"]
    for s in ORDER:
        py.append("    %r: (%d, {" % (s, sizes[s]))
        for ctype, name in MEMBERS[s]:
            py.append("        %r: (%d, %r)," % (name, offs[(s, name)], ctype))
        py.append("    }),")
    py.append("}")
    return "\n".join(h) + "\n", "\n".join(py) + "\n"


def main(argv):
    check = "--check" in argv
    args = [a for a in argv if not a.startswith("--")]
    src = args[0] if args else os.environ.get("MDZ_REF_SRC", "/root/reference/SOURCE")
    header, py = render(*measure(src))
    if check:
        ok = open(HEADER_OUT).read() == header and open(PY_OUT).read() == py
        print("layout up to date" if ok else "layout differs from the reference header")
        return 0 if ok else 1
    with open(HEADER_OUT, "w") as fh:
        fh.write(header)
    with open(PY_OUT, "w") as fh:
        fh.write(py)
    print("wrote", HEADER_OUT, PY_OUT)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
