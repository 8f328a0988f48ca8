"""Build recipe for oracle/_ref: the reference's own SR kernels (TEST
INFRASTRUCTURE ONLY).

Compiles oracle/ref_entity.cpp, which includes Entity's kernel headers where
they lie in the reference checkout (src/kernels/pushers/sr.hpp, gr.hpp,
currents_deposit.hpp, particle_shapes.hpp, faraday_mink.hpp, ampere_mink.hpp,
digital_filter.hpp, faraday_gr.hpp, ampere_gr.hpp, aux_fields_gr.hpp,
fields_bcs.hpp, src/metrics/minkowski.h, qkerr_schild.h,
src/global/utils/sorting.h and what they include), against the host Kokkos
shim in oracle/kokkos_shim.
Nothing is copied: the headers are read in place through -I. The reference's
own build system (cmake with Kokkos 5.0.1, an empty submodule here) is not
used.

One library per precision and shape order, because the reference fixes both
at compile time (cmake/config.cmake:4-28; order 0, the zigzag deposit, leaves
SHAPE_ORDER undefined):
  oracle/_ref/libentity_ref_{f32,f64}_o{0,1,2,3}.so
g++ -std=c++20 -O2 -ffp-contract=off: no contraction, so every product and
sum rounds as the reference's source writes it. OpenMP splits each
parallel_for statically over the threads, and the scatter view of the
current deposit keeps one copy per thread, summed in thread order at
contribute(): the same partition and summation order as the oracle's
deposit, so the two give the same J bit for bit.

A second library per precision, oracle/_ref/libentity_ref_params_{f32,f64}.so,
compiles oracle/ref_params.cpp with the reference's parameter sources
(src/framework/parameters/*.cpp, src/global/utils/param_container.cpp,
src/global/arch/kokkos_aliases.cpp) to run its own TOML-to-scales derivation.
A third, oracle/_ref/libentity_ref_particles_{f32,f64}.so, compiles
oracle/ref_particles.cpp with the reference's particle container and grid
(src/framework/containers/particles.cpp, particles_sort.cpp,
src/framework/domain/grid.cpp) to run its own RemoveDead, SortSpatially and
the output moments of ParticleMoments_kernel on that container.

The reference checkout is located by $ENTITY_REFERENCE, else
/root/reference. Without it, build() returns {} and the tests that need these
libraries skip.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(HERE, "ref_entity.cpp")
SHIM = os.path.join(HERE, "kokkos_shim")


def reference_root():
    root = os.environ.get("ENTITY_REFERENCE", "/root/reference")
    return root if os.path.isfile(os.path.join(root, "src", "kernels", "pushers", "sr.hpp")) else None


def _deps(root):
    deps = [SRC, os.path.join(HERE, "srpic_oracle.h")]
    deps += [os.path.join(SHIM, f) for f in os.listdir(SHIM)]
    return deps


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _flags(root):
    return ["-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            "-fopenmp", "-DENTITY_SHIM_OPENMP", "-w", "-I", SHIM, "-I", HERE, "-I", os.path.join(root, "src"),
            "-I", os.path.join(root, "src", "global"), "-I", os.path.join(root, "include")]


def build(verbose=False, jobs=None):
    root = reference_root()
    if root is None:
        return {}
    os.makedirs(OUT, exist_ok=True)
    deps = _deps(root)
    todo, libs = [], {}
    for tag, defs in (("f32", ["-DSINGLE_PRECISION"]), ("f64", [])):
        for order in range(4):
            target = os.path.join(OUT, f"libentity_ref_{tag}_o{order}.so")
            libs[(tag, order)] = target
            if _stale(target, deps):
                # the zigzag deposit leaves SHAPE_ORDER undefined (order 0,
                # N_GHOSTS = 2); Esirkepov sets it (cmake/config.cmake:20-28)
                so = [f"-DSHAPE_ORDER={order}"] if order > 0 else []
                todo.append(["g++", *_flags(root), *defs, *so, SRC, "-o", target])

    psrc = [os.path.join(HERE, "ref_params.cpp")]
    pdir = os.path.join(root, "src", "framework", "parameters")
    psrc += sorted(os.path.join(pdir, f) for f in os.listdir(pdir) if f.endswith(".cpp"))
    psrc += [os.path.join(root, "src", "global", "utils", "param_container.cpp"),
             os.path.join(root, "src", "global", "arch", "kokkos_aliases.cpp")]
    for tag, defs in (("f32", ["-DSINGLE_PRECISION"]), ("f64", [])):
        target = os.path.join(OUT, f"libentity_ref_params_{tag}.so")
        libs[("params", tag)] = target
        if _stale(target, deps + psrc[:1]):
            todo.append(["g++", *_flags(root), "-O1", *defs, *psrc, "-o", target])

    # the reference's particle container and grid, for its own sort
    # (Particles::RemoveDead and SortSpatially) and output moments, driven by
    # oracle/ref_particles.cpp
    ssrc = [os.path.join(HERE, "ref_particles.cpp")]
    ssrc += [os.path.join(root, "src", "framework", "containers", f)
             for f in ("particles.cpp", "particles_sort.cpp")]
    ssrc += [os.path.join(root, "src", "framework", "domain", "grid.cpp"),
             os.path.join(root, "src", "global", "arch", "kokkos_aliases.cpp")]
    for tag, defs in (("f32", ["-DSINGLE_PRECISION"]), ("f64", [])):
        target = os.path.join(OUT, f"libentity_ref_particles_{tag}.so")
        libs[("particles", tag)] = target
        if _stale(target, deps + ssrc[:1]):
            todo.append(["g++", *_flags(root), "-O1", *defs, *ssrc, "-o", target])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, todo))
    return libs


# the reference's own kernel tests (tests/kernels/*.cpp, main() programs that
# throw on a mismatch) for the hot path's kernels; they run against the shim
KERNEL_TESTS = ["deposit", "pusher", "gca_pusher", "ext_force", "prtl_bc", "faraday_mink",
                "ampere_mink", "digital_filter", "fields_to_phys", "prtls_to_phys", "flds_bc"]
# the reference's metric tests (tests/metrics/*.cpp): QKerrSchild against
# Kerr-Schild at h = 0, 0.1 and 0.25, coordinate and vector transformations
METRIC_TESTS = ["ks-qks", "ks-qks-4d", "coord_trans", "vec_trans"]
# and its framework tests with the sources they link: the bin sort of a key
# (tests/global/sorting.cpp), the tile index (tiling.cpp), the particle
# container and its spatial sort (tests/framework/particles.cpp,
# particles_sort.cpp), the field container (fields.cpp) and the single-domain
# field exchange (comm-nompi.cpp)
LINKED_TESTS = {
    "sorting": ("global", ["src/global/global.cpp"]),
    "tiling": ("global", ["src/global/global.cpp"]),
    "particles": ("framework", ["src/global/global.cpp",
                                "src/framework/containers/particles.cpp"]),
    "particles_sort": ("framework", ["src/global/global.cpp",
                                     "src/framework/containers/particles.cpp",
                                     "src/framework/containers/particles_sort.cpp",
                                     "src/framework/domain/grid.cpp"]),
    "fields": ("framework", ["src/global/global.cpp",
                             "src/framework/containers/fields.cpp"]),
    "comm-nompi": ("framework", ["src/global/global.cpp"]),
}


def build_tests(verbose=False, jobs=None):
    """Compiles the reference's kernel, metric and framework tests unmodified
    against the shim into oracle/_ref/tests/<name>_{f32,f64}; returns
    {(name, tag): path}."""
    root = reference_root()
    if root is None:
        return {}
    tdir = os.path.join(OUT, "tests")
    os.makedirs(tdir, exist_ok=True)
    deps = _deps(root)
    aliases = os.path.join(root, "src", "global", "arch", "kokkos_aliases.cpp")
    todo, exes = [], {}
    for name in KERNEL_TESTS + METRIC_TESTS + list(LINKED_TESTS):
        extra = []
        if name in LINKED_TESTS:
            sub, rel = LINKED_TESTS[name]
            extra = [os.path.join(root, r) for r in rel]
        else:
            sub = "kernels" if name in KERNEL_TESTS else "metrics"
        src = os.path.join(root, "tests", sub, name + ".cpp")
        for tag, defs in (("f32", ["-DSINGLE_PRECISION"]), ("f64", [])):
            target = os.path.join(tdir, f"{name}_{tag}")
            exes[(name, tag)] = target
            if _stale(target, deps + [src]):
                flags = [f for f in _flags(root) if f not in ("-shared", "-fPIC")]
                todo.append(["g++", *flags, "-O1", *defs, src, *extra, aliases, "-o", target])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, todo))
    return exes


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    if "--tests" in sys.argv:
        print(build_tests(verbose="-v" in sys.argv))
