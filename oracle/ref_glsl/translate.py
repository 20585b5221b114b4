"""Mechanical GLSL -> C++ rewrite of the reference's compute shaders and of its
sky-rendering headers.

TEST INFRASTRUCTURE ONLY (oracle pinning). Reads the reference's shader
sources where they lie (shaders/util.h, params.h, transmittance.h,
irradiance.h, scattering.h, the six precompute *.comp files, render_sky.h and
render_lighting.h) and writes
compilable C++ copies into oracle/_ref/gen/ (git-ignored), never into the
repository. The rewrite is purely syntactic, so the arithmetic compiled is the
reference's own:

  * '#version' and 'layout(local_size...) in;' lines are dropped;
  * 'layout(...) uniform Block { decls };' becomes the bare declarations
    (uniform block members are globals of the pass);
  * 'layout(...) uniform [writeonly] sampler/image NAME;' becomes a global;
  * 'out T name' parameters become 'T& name';
  * swizzles '.rgb' / '.xy' become member calls;
  * 'void main()' becomes 'void main_entry(uvec3 gl_GlobalInvocationID)'.

Built-ins, vector types, samplers and images come from glsl_shim.hpp.
"""
import argparse
import os
import re
import sys

HEADERS = ["util.h", "params.h", "transmittance.h", "irradiance.h", "scattering.h"]
# the renderer's shading functions (render_sky.frag includes render_sky.h)
RENDER = ["render_sky.h", "render_lighting.h"]
PASSES = [
    "transmittance.comp",
    "direct_irradiance.comp",
    "single_scattering.comp",
    "scattering_density.comp",
    "indirect_irradiance.comp",
    "multiple_scattering.comp",
]


def rewrite(src: str) -> str:
    out = re.sub(r"^\s*#version[^\n]*\n", "", src, flags=re.M)
    out = re.sub(r"^\s*layout\s*\([^)]*\)\s*in\s*;[^\n]*\n", "", out, flags=re.M)
    # uniform / push-constant blocks -> their member declarations
    out = re.sub(
        r"layout\s*\([^)]*\)\s*uniform\s+\w+\s*\{([^}]*)\}\s*;",
        lambda m: m.group(1).strip(),
        out,
    )
    # opaque uniforms -> globals
    out = re.sub(
        r"layout\s*\([^)]*\)\s*uniform\s+(?:(?:writeonly|readonly)\s+)*(\w+)\s+(\w+)\s*;",
        r"\1 \2;",
        out,
    )
    out = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", out)
    out = re.sub(r"\.rgb\b", ".rgb()", out)
    out = re.sub(r"\.xy\b", ".xy()", out)
    out = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void main_entry(uvec3 gl_GlobalInvocationID)", out)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--shaders", required=True, help="the reference's shaders/ directory")
    ap.add_argument("--out", required=True, help="output directory (oracle/_ref/gen)")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    for name in HEADERS + PASSES + RENDER:
        with open(os.path.join(a.shaders, name)) as f:
            text = f.read()
        with open(os.path.join(a.out, name), "w") as f:
            f.write("// generated by oracle/ref_glsl/translate.py; do not commit\n")
            f.write(rewrite(text))
    return 0


if __name__ == "__main__":
    sys.exit(main())
