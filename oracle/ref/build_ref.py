#!/usr/bin/env python3
"""Builds oracle/_ref/libref.so: the reference's own step kernels (physics/ocl/kernels/*.cl
of axoloto/RealTimeParticles) and its Perlin noise (physics/utils/PerlinNoise.cpp) compiled
for the CPU, to check the oracle against them.

TEST INFRASTRUCTURE ONLY.  When the reference checkout is present (REFERENCE_DIR, default: a
checkout named `reference` next to this repository), each OpenCL program is assembled from its .cl files in the order the
reference's createProgram uses (Fluids.cpp:123, Boids.cpp:117, Clouds.cpp:157), the OpenCL
vector literals "(float4)(a, b, ...)" are rewritten to "make_float4(a, b, ...)" (the only
change: C++ would read them as comma expressions), and the result is written to
oracle/_ref/ref_<program>.cpp inside its own namespace, with the JIT -D constants bound to
a runtime struct.  Everything generated stays in oracle/_ref/ (git-ignored).  When only the
generated sources are present (no checkout), they are compiled as they are.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
REF = os.environ.get("REFERENCE_DIR", os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference"))
KDIR = os.path.join(REF, "physics", "ocl", "kernels")

PROGRAMS = {
    "fluids": ["define.cl", "sph.cl", "fluids.cl", "utils.cl", "grid.cl"],
    "boids": ["define.cl", "boids.cl", "utils.cl", "grid.cl"],
    "clouds": ["define.cl", "sph.cl", "clouds.cl", "grid.cl", "utils.cl"],
}

# The -D constants of the reference's JIT programs (Fluids.cpp:104-119, Boids.cpp:103-113,
# Clouds.cpp:134-147), bound to rtp_grid_constants set by the driver before each call.
DEFINES = {
    "EFFECT_RADIUS": "(ref_consts.effectRadius)",
    "EFFECT_RADIUS_SQUARED": "(ref_consts.effectRadiusSquared)",
    "ABS_WALL_X": "(ref_consts.absWall[0])",
    "ABS_WALL_Y": "(ref_consts.absWall[1])",
    "ABS_WALL_Z": "(ref_consts.absWall[2])",
    "GRID_RES_X": "((int)ref_consts.gridRes[0])",
    "GRID_RES_Y": "((int)ref_consts.gridRes[1])",
    "GRID_RES_Z": "((int)ref_consts.gridRes[2])",
    "GRID_CELL_SIZE_XYZ": "(ref_consts.cellSize)",
    "GRID_NUM_CELLS": "((int)ref_consts.numCells)",
    "NUM_MAX_PARTS_IN_CELL": "((int)ref_consts.maxPartsInCell)",
    "POLY6_COEFF": "(ref_consts.poly6Coeff)",
    "SPIKY_COEFF": "(ref_consts.spikyCoeff)",
    "MAX_VEL": "(ref_consts.maxVel)",
}

LITERAL = re.compile(r"\((float|int|uint)([2348])\)\s*\(")


def generate():
    os.makedirs(OUT, exist_ok=True)
    for prog, files in PROGRAMS.items():
        body = []
        for f in files:
            src = open(os.path.join(KDIR, f)).read()
            src = LITERAL.sub(r"make_\1\2(", src)
            # ".xyz" of a float3 is the float3 itself (utils.cl fillCameraDist, render-only).
            src = src.replace("cameraPos[0].xyz", "cameraPos[0]")
            body.append("// ---- %s\n#line 1 \"%s\"\n%s\n" % (f, f, src))
        defs = "\n".join("#define %s %s" % kv for kv in DEFINES.items())
        undefs = "\n".join("#undef %s" % k for k in DEFINES)
        text = ("// Generated by oracle/ref/build_ref.py from %s (OpenCL vector literals rewritten).\n"
                "#include \"../ref/clshim.hpp\"\n#include \"../../include/rtp.h\"\n"
                "extern rtp_grid_constants ref_consts;\n"
                "namespace ref_%s {\nusing namespace clshim;\n%s\n%s\n%s\n}  // namespace ref_%s\n"
                % (", ".join(files), prog, defs, "".join(body), undefs, prog))
        open(os.path.join(OUT, "ref_%s.cpp" % prog), "w").write(text)
    # Physics::PerlinNoise (the boids target's noise) and the math header it includes, as
    # they are: they compile alone.  Target.cpp needs spdlog and nlohmann/json (absent).
    pdir = os.path.join(OUT, "perlin")
    os.makedirs(pdir, exist_ok=True)
    for src in (os.path.join(REF, "physics", "utils", "PerlinNoise.cpp"),
                os.path.join(REF, "physics", "utils", "PerlinNoise.hpp"),
                os.path.join(REF, "utils", "Math.hpp")):
        open(os.path.join(pdir, os.path.basename(src)), "w").write(open(src).read())
    # Geometry's reset-case lattices (utils/Geometry.cpp) with the headers it includes, as they
    # are, except Logging.hpp (spdlog, absent): a two-line stand-in that drops the log calls.
    gdir = os.path.join(OUT, "geometry")
    os.makedirs(gdir, exist_ok=True)
    for src in (os.path.join(REF, "utils", "Geometry.cpp"), os.path.join(REF, "utils", "Geometry.hpp"),
                os.path.join(REF, "utils", "Math.hpp")):
        open(os.path.join(gdir, os.path.basename(src)), "w").write(open(src).read())
    open(os.path.join(gdir, "Logging.hpp"), "w").write(
        "#pragma once\n#define LOG_ERROR(...) ((void)0)\n")


def compile_lib():
    gen = [os.path.join(OUT, "ref_%s.cpp" % p) for p in PROGRAMS]
    if not all(os.path.exists(s) for s in gen):
        return False
    out = os.path.join(OUT, "libref.so")
    # The driver includes the generated programs (one namespace each) into one unit.
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-I", OUT, "-shared", "-o", out, os.path.join(HERE, "ref_driver.cpp"),
           os.path.join(HERE, "ref_geometry.cpp")]
    subprocess.run(cmd, check=True)
    return True


def main():
    if os.path.isdir(KDIR):
        generate()
    ok = compile_lib()
    if not ok:
        print("oracle/_ref: reference kernels not available (no checkout, no generated sources)", file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
