"""Build recipe for the reference (Athena++) binaries used to pin the oracle.

Test infrastructure only: nothing in the product imports or runs this.

The reference's own build (``configure.py`` -> ``Makefile``/``src/defs.hpp``) writes
into its source tree, which is read-only here, so this recipe does the same two steps
itself without touching the tree:

* it fills the reference's ``src/defs.hpp.in`` template with the macro values that
  ``configure.py -b --flux=<f> [--nghost=3] [-s]`` would choose (configure.py:451-560)
  and writes the result to ``oracle/_ref/<variant>/gen/defs.hpp``;
* it compiles the same source list as ``Makefile.in:29-75`` with ``g++ -O3 -std=c++11``
  (the flags configure.py uses for g++, configure.py:560-566) straight from the
  reference's ``src/`` into ``oracle/_ref/<variant>/obj`` and links two executables:
  ``athena_lw`` (the reference's own ``pgen/linear_wave.cpp``), ``athena_blast`` (its
  own ``pgen/blast.cpp``, used for the multi-level cases), ``athena_ic``
  (``oracle/ref_pgen/load_ic.cpp``) and ``athena_blocks``
  (``oracle/ref_pgen/load_blocks.cpp``, per-block initial states of multi-level meshes),
  all with ``oracle/ref_pgen/dump_hook.cpp``.

Nothing is copied out of the reference tree; all outputs go under ``oracle/_ref/``.
Usage: ``python oracle/build_ref.py [variant ...]`` (default: all variants).
"""
import glob
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

REF = os.environ.get("ATHENA_REF_SRC", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def reference_present():
    """True where the reference's source tree is available (this recipe can build)."""
    return os.path.isdir(os.path.join(REF, "src"))
OUT = os.path.join(HERE, "_ref")

# variant -> (riemann solver, nghost, relativistic)
VARIANTS = {
    "mhd_hlld_g2": ("hlld", 2, False),
    "mhd_hlld_g3": ("hlld", 3, False),
    "mhd_hlle_g2": ("hlle", 2, False),
    "mhd_hlle_g3": ("hlle", 3, False),
    "mhd_hlld_g4": ("hlld", 4, False),   # PPM with mesh refinement (even NGHOST)
    "mhd_llf_g2": ("llf", 2, False),     # local Lax-Friedrichs (llf_mhd.cpp)
    "mhd_roe_g2": ("roe", 2, False),     # Roe linearisation (roe_mhd.cpp)
    "mhd_lhlld_g2": ("lhlld", 2, False),  # low-dissipation HLLD (lhlld.cpp)
    "mhd_lhlld_g3": ("lhlld", 3, False),
    "srmhd_hlle_g2": ("hlle", 2, True),
    "srmhd_llf_g2": ("llf", 2, True),    # relativistic LLF (llf_mhd_rel.cpp)
    "srmhd_hlld_g2": ("hlld", 2, True),  # relativistic HLLD (hlld_rel.cpp)
}


def defs_values(flux, ng, sr):
    return {
        "PROBLEM": "linear_wave", "COORDINATE_SYSTEM": "cartesian", "RSOLVER": flux,
        "EQUATION_OF_STATE": "adiabatic",
        "CHEMNETWORK_HEADER": "../chemistry/network/chem_network.hpp",
        "CHEMRADIATION_INTEGRATOR": "none", "GENERAL_EOS": "0", "EOS_TABLE_ENABLED": "0",
        "NON_BAROTROPIC_EOS": "1", "MAGNETIC_FIELDS_ENABLED": "1", "STS_ENABLED": "0",
        "SELF_GRAVITY_ENABLED": "0", "CHEMISTRY_ENABLED": "0",
        "CHEMRADIATION_ENABLED": "0", "NR_RADIATION_ENABLED": "0",
        "IM_RADIATION_ENABLED": "0", "CR_ENABLED": "0", "CRDIFFUSION_ENABLED": "0",
        "RELATIVISTIC_DYNAMICS": "1" if sr else "0", "GENERAL_RELATIVITY": "0",
        "SINGLE_PRECISION_ENABLED": "0", "H5_DOUBLE_PRECISION_ENABLED": "0",
        "DEBUG_OPTION": "0", "FFT_OPTION": "NO_FFT", "MPI_OPTION": "NOT_MPI_PARALLEL",
        "OPENMP_OPTION": "NOT_OPENMP_PARALLEL", "HDF5_OPTION": "NO_HDF5OUTPUT",
        "CVODE_OPTION": "NO_CVODE", "EXCEPTION_HANDLING_OPTION": "ENABLE_EXCEPTIONS",
        "COMPILER_CHOICE": "g++", "COMPILER_COMMAND": "g++",
        "COMPILER_FLAGS": "-O3 -std=c++11", "NHYDRO_VARIABLES": "5",
        "NFIELD_VARIABLES": "3", "NWAVE_VALUE": "7", "NUMBER_PASSIVE_SCALARS": "0",
        "NUMBER_CHEMICAL_SPECIES": "0", "NUMBER_GHOST_CELLS": str(ng),
        "NCR_VARIABLES": "0", "NRAD_VARIABLES": "0",
    }


def source_list(flux, sr):
    s = os.path.join(REF, "src")
    files = []
    for d in ["", "bvals", "bvals/cc", "bvals/cc/fft_grav", "bvals/cc/hydro", "bvals/cc/mg",
              "bvals/cc/nr_radiation", "bvals/fc", "bvals/orbital", "bvals/sixray",
              "bvals/utils", "chem_rad", "fft", "field", "field/field_diffusion",
              "gravity", "hydro", "hydro/srcterms", "hydro/hydro_diffusion",
              "nr_radiation", "nr_radiation/integrators",
              "nr_radiation/integrators/srcterms", "nr_radiation/implicit", "cr",
              "cr/integrators", "crdiffusion", "inputs", "mesh", "multigrid",
              "orbital_advection", "outputs", "reconstruct", "scalars", "task_list",
              "utils", "units", "chemistry/utils"]:
        files += sorted(glob.glob(os.path.join(s, d, "*.cpp")))
    eos = "adiabatic_mhd_sr.cpp" if sr else "adiabatic_mhd.cpp"
    # configure.py:476-531: hlle/llf/roe get "_mhd", then "_rel" for -s
    rs = flux + ("_mhd" if flux in ("hlle", "llf", "roe") else "") + \
        ("_rel" if sr else "") + ".cpp"
    files += [
        os.path.join(s, "coordinates/coordinates.cpp"),
        os.path.join(s, "coordinates/cartesian.cpp"),
        os.path.join(s, "eos", eos),
        os.path.join(s, "eos/general/noop.cpp"),  # GENERAL_EOS_FILE (configure.py:462)
        os.path.join(s, "eos/eos_high_order.cpp"),
        os.path.join(s, "eos/eos_scalars.cpp"),
        os.path.join(s, "chemistry/network_wrapper.cpp"),
        os.path.join(s, "chemistry/network/none.cpp"),
        os.path.join(s, "chemistry/forward_euler.cpp"),
        os.path.join(s, "chem_rad/integrators/const.cpp"),
        os.path.join(s, "hydro/rsolvers/mhd", rs),
        os.path.join(s, "pgen/default_pgen.cpp"),
    ]
    return files


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))


def build_variant(name, jobs=None):
    flux, ng, sr = VARIANTS[name]
    vdir = os.path.join(OUT, name)
    gen, obj = os.path.join(vdir, "gen"), os.path.join(vdir, "obj")
    os.makedirs(gen, exist_ok=True)
    os.makedirs(obj, exist_ok=True)
    tmpl = open(os.path.join(REF, "src/defs.hpp.in")).read()
    for k, v in defs_values(flux, ng, sr).items():
        tmpl = re.sub(r"@%s@" % k, v, tmpl)
    defs = os.path.join(gen, "defs.hpp")
    if not os.path.exists(defs) or open(defs).read() != tmpl:
        with open(defs, "w") as f:
            f.write(tmpl)
    # the sources include the configured header as "defs.hpp", "../defs.hpp",
    # "../../defs.hpp" and "../../../../defs.hpp"; give each form a search directory
    # that resolves to gen/defs.hpp
    deep = os.path.join(gen, "a", "b", "c", "d")
    os.makedirs(deep, exist_ok=True)
    cxx = ["g++", "-O3", "-std=c++11", "-ffp-contract=off", "-I", gen,
           "-I", os.path.join(gen, "a"), "-I", os.path.join(gen, "a", "b"), "-I", deep,
           "-I", os.path.join(REF, "src")]
    srcs = source_list(flux, sr)
    extra = {"dump_hook": os.path.join(HERE, "ref_pgen/dump_hook.cpp"),
             "load_ic": os.path.join(HERE, "ref_pgen/load_ic.cpp"),
             "linear_wave": os.path.join(REF, "src/pgen/linear_wave.cpp"),
             "blast": os.path.join(REF, "src/pgen/blast.cpp"),
             "load_blocks": os.path.join(HERE, "ref_pgen/load_blocks.cpp")}

    def objname(src):
        rel = os.path.relpath(src, REF).replace("/", "_") if src.startswith(REF) else \
            os.path.basename(src)
        return os.path.join(obj, rel[:-4] + ".o")

    def compile_one(src):
        o = objname(src)
        if os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(src),
                                                            os.path.getmtime(defs)):
            return o
        run(cxx + ["-c", src, "-o", o])
        return o

    with ThreadPoolExecutor(jobs or os.cpu_count()) as ex:
        objs = list(ex.map(compile_one, srcs))
        eobj = dict(zip(extra, ex.map(compile_one, extra.values())))
    for exe, pg in (("athena_lw", "linear_wave"), ("athena_ic", "load_ic"),
                    ("athena_blast", "blast"), ("athena_blocks", "load_blocks")):
        if sr and pg in ("linear_wave", "blast", "load_blocks"):
            continue
        run(cxx + ["-o", os.path.join(vdir, exe)] + objs + [eobj[pg], eobj["dump_hook"]])
    return vdir


# The reference with the library's per-operator shim (athena_gb300/shim/): the member
# functions the shim defines, and the reference object files that define them
SHIM = os.path.join(os.path.dirname(HERE), "athena_gb300", "shim", "athgpu_operator_shim.cpp")
SHIM_REPLACES = {
    "src_hydro_calculate_fluxes.o": "Hydro::CalculateFluxes(",
    "src_hydro_add_flux_divergence.o": "Hydro::AddFluxDivergence(",
    "src_hydro_new_blockdt.o": "Hydro::NewBlockTimeStep(",
    "src_field_calculate_corner_e.o": "Field::ComputeCornerE(",
    "src_field_ct.o": "Field::CT(",
    "src_eos_adiabatic_mhd.o": "EquationOfState::ConservedToPrimitive(",
}


def defined_symbols(obj):
    """(mangled, demangled) names of the functions an object file defines (nm of an
    object compiled here from the reference's sources)."""
    raw = subprocess.run(["nm", "--defined-only", obj], capture_output=True, text=True,
                         check=True).stdout.splitlines()
    dem = subprocess.run(["nm", "-C", "--defined-only", obj], capture_output=True, text=True,
                         check=True).stdout.splitlines()
    out = []
    for a, b in zip(raw, dem):
        pa, pb = a.split(None, 2), b.split(None, 2)
        if len(pa) == 3 and pa[1] in "TtWw":
            out.append((pa[2], pb[2]))
    return out


def build_gpu_variant(base="mhd_hlld_g2", lib_dir=None):
    """The reference linked with the operator shim: the base variant's objects, the six
    replaced member functions made weak (objcopy --weaken-symbol) so that the shim's
    definitions take their place, the shim compiled against the reference's headers and
    this repository's include/, linked with libathgpu.so.  Writes
    oracle/_ref/<base>_gpu/athena_lw (the reference's linear_wave problem generator and
    the state dump hook).  Needs libathgpu.so built (athena_gb300/build.py)."""
    flux, ng, sr = VARIANTS[base]
    bdir = build_variant(base)
    vdir = os.path.join(OUT, base + "_gpu")
    wobj = os.path.join(vdir, "obj")
    os.makedirs(wobj, exist_ok=True)
    repo = os.path.dirname(HERE)
    lib_dir = lib_dir or os.path.join(repo, "athena_gb300")
    gen = os.path.join(bdir, "gen")
    cxx = ["g++", "-O3", "-std=c++11", "-ffp-contract=off", "-I", gen,
           "-I", os.path.join(gen, "a"), "-I", os.path.join(gen, "a", "b"),
           "-I", os.path.join(gen, "a", "b", "c", "d"), "-I", os.path.join(REF, "src"),
           "-I", os.path.join(repo, "include")]
    objs = []
    for o in sorted(glob.glob(os.path.join(bdir, "obj", "src_*.o"))):
        name = os.path.basename(o)
        if name.startswith("src_pgen_") and name != "src_pgen_default_pgen.o":
            continue
        if name in SHIM_REPLACES:
            want = SHIM_REPLACES[name]
            syms = [m for m, d in defined_symbols(o) if d.startswith(want)]
            if len(syms) != 1:
                raise RuntimeError("%s: %d definitions of %s" % (name, len(syms), want))
            w = os.path.join(wobj, name)
            run(["objcopy", "--weaken-symbol=" + syms[0], o, w])
            objs.append(w)
        else:
            objs.append(o)
    shim_o = os.path.join(wobj, "athgpu_operator_shim.o")
    run(cxx + ["-c", SHIM, "-o", shim_o])
    extra = [os.path.join(bdir, "obj", "src_pgen_linear_wave.o"),
             os.path.join(bdir, "obj", "dump_hook.o")]
    exe = os.path.join(vdir, "athena_lw")
    cuda_lib = "/usr/local/cuda/lib64"
    run(cxx + ["-o", exe] + objs + [shim_o] + extra +
        ["-L", lib_dir, "-lathgpu", "-Wl,-rpath," + lib_dir, "-L", cuda_lib,
         "-Wl,-rpath-link," + cuda_lib, "-lcudart"])
    return exe


def main(argv):
    names = argv or list(VARIANTS)
    for n in names:
        print("building", n, "->", build_variant(n), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
