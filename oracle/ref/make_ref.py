#!/usr/bin/env python3
"""Build oracle/_ref/libgrisref.so, libdiref.so and libpostref.so: the reference's own GRIS,
ReSTIR DI and presentation (post_proc.frag) shader code, compiled as C++.

TEST INFRASTRUCTURE (oracle). The output is the pinning reference for the oracle
restatement; it is never part of the product and never travels as source.

Recipe
------
1. Read the reference's shader sources where they lie (REFERENCE/src/shader/*.glsl and
   HostDevice.h). Nothing is copied into the repository: the rewritten files go to
   oracle/_ref/glsl/, which is git-ignored.
2. Apply a mechanical GLSL -> C++20 rewrite (no edits by hand):
   - HostDevice.h: take the shader-side branch of its `#ifdef __cplusplus`.
   - `layout(...) uniform|buffer _Block { members };` -> the members as globals, an
     unsized array `T a[];` becoming `GBuf<T> a;` (a bounds-checked buffer view);
     `layout(...) uniform sampler2D x;` -> `sampler2D x;`; a fragment shader's
     `layout(location = n) in|out T x;` -> the global `T x;`.
   - `out T x` / `inout T x` parameters -> `T& x`.
   - swizzles .xy .zw .yz .xyz .yzw .rgb -> accessor calls returning references.
   - vector constructors whose arguments draw random numbers (`sampleNf(...)`) use
     braces, so C++ evaluates the draws left to right as GLSL requires.
   - `#pragma unroll` lines are dropped.
   - the hard-coded path depth (`MaxTracingDepth = 15`), spatial neighbour count
     (`ResampleNum = 3`) and radius (`ResampleRadius = 20.0`) become run-time
     parameters whose defaults are the reference's values.
3. Compile oracle/ref/alias_ref.cpp against the reference's src/util/AliasTable.h (plain
   C++, used as is) into oracle/_ref/libaliasref.so.
4. Compile oracle/ref/ref_harness.cpp (the GRIS pass), oracle/ref/ref_harness_di.cpp
   (the ReSTIR DI pass) and oracle/ref/ref_harness_post.cpp (the presentation pass), each
   including the rewritten shaders after glsl_compat.h and ref_common.h, with g++ -std=c++20
   -fsingle-precision-constant -ffp-contract=off -ftrivial-auto-var-init=zero -fopenmp, into
   oracle/_ref/libgrisref.so, libdiref.so and libpostref.so.

Usage: python oracle/ref/make_ref.py [--reference DIR] [--out DIR]
The reference sources are looked up in --reference, else $GRIS_REFERENCE, else the checkout
location below; where none holds them the recipe builds nothing and exits with status 2.
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
DEFAULT_REF = "/root/reference"

SHADERS = [
    "HostDevice.h", "layouts.glsl", "ray_layouts.glsl", "math.glsl", "material.glsl",
    "camera.glsl", "gbuffer_util.glsl", "ray_gbuffer_util.glsl", "light_sampling.glsl",
    "gris_reservoir.glsl", "gris_path_trace.glsl", "gris_retrace.glsl",
    "gris_resample_temporal.glsl", "gris_resample_spatial.glsl", "gi_naive.glsl",
    "di_reservoir.glsl", "di_path_gen.glsl", "di_temporal.glsl", "di_spatial.glsl",
    "post_proc.frag",
]


def _match_paren(s, i, open_c="(", close_c=")"):
    depth = 0
    for j in range(i, len(s)):
        if s[j] == open_c:
            depth += 1
        elif s[j] == close_c:
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced at %d" % i)


def _rewrite_decl(decl):
    """`uniform _Camera { Camera uCamera; ... };` -> member globals; plain uniforms kept."""
    decl = decl.strip()
    decl = re.sub(r"\b(readonly|writeonly|uniform|buffer|coherent|restrict)\b\s*", "", decl)
    if "{" in decl:
        body = decl[decl.index("{") + 1: decl.rindex("}")]
        out = []
        for m in body.split(";"):
            m = m.strip()
            if not m:
                continue
            am = re.match(r"^(\w+)\s+(\w+)\s*\[\s*\]$", m)
            out.append("GBuf<%s> %s;" % (am.group(1), am.group(2)) if am else m + ";")
        return "\n".join(out)
    decl = re.sub(r"^(in|out)\s+", "", decl)   # a fragment shader's interface variable -> a global
    am = re.match(r"^(\w+)\s+(\w+)\s*\[\s*\]\s*;$", decl)
    if am:
        return "GBuf<%s> %s;" % (am.group(1), am.group(2))
    return decl


def _rewrite_layouts(src):
    out, i = [], 0
    while True:
        k = src.find("layout(", i)
        if k < 0:
            out.append(src[i:])
            break
        out.append(src[i:k])
        p = _match_paren(src, k + len("layout"))
        j = p + 1
        semi = src.find(";", j)
        brace = src.find("{", j)
        if 0 <= brace < semi:
            close = _match_paren(src, brace, "{", "}")
            semi = src.find(";", close)
        decl = src[j:semi + 1]
        out.append(_rewrite_decl(decl))
        i = semi + 1
    return "".join(out)


def _brace_rng_ctors(src):
    """vecN(...sampleNf(...)...) -> vecN{...}: braced lists evaluate left to right."""
    out, i = [], 0
    pat = re.compile(r"\b(vec[234])\(")
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            break
        open_i = m.end() - 1
        close_i = _match_paren(src, open_i)
        inner = src[open_i + 1:close_i]
        out.append(src[i:m.start()])
        if re.search(r"\bsample[1-4]f\s*\(", inner):
            out.append("%s{%s}" % (m.group(1), _brace_rng_ctors(inner)))
        else:
            out.append("%s(%s)" % (m.group(1), _brace_rng_ctors(inner)))
        i = close_i + 1
    return "".join(out)


def rewrite(name, src):
    if name == "HostDevice.h":
        return src.replace("#ifdef __cplusplus", "#if 0 /* shader-side branch */", 1)
    src = "\n".join(l for l in src.split("\n")
                    if not re.match(r"\s*#\s*(version|extension|pragma\s+unroll)\b", l))
    src = _rewrite_layouts(src)
    src = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", src)
    src = re.sub(r"\.(xyz|yzw|rgb|xy|zw|yz)\b", r".\1()", src)
    src = _brace_rng_ctors(src)
    src = re.sub(r"const\s+int\s+MaxTracingDepth\s*=\s*15\s*;",
                 "const int MaxTracingDepth = GREF_MAX_DEPTH;", src)
    src = re.sub(r"const\s+uint\s+ResampleNum\s*=\s*3\s*;",
                 "const uint ResampleNum = GREF_RESAMPLE_NUM;", src)
    src = re.sub(r"const\s+float\s+ResampleRadius\s*=\s*20\.0\s*;",
                 "const float ResampleRadius = GREF_RESAMPLE_RADIUS;", src)
    return src


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("GRIS_REFERENCE", DEFAULT_REF))
    ap.add_argument("--out", default=os.path.join(ORACLE, "_ref"))
    ap.add_argument("--cxx", default=os.environ.get("CXX", "g++"))
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args()
    shader_dir = os.path.join(args.reference, "src", "shader")
    if not os.path.isdir(shader_dir):
        print("reference shaders not found at %s; oracle/_ref not built" % shader_dir)
        return 2
    gdir = os.path.join(args.out, "glsl")
    os.makedirs(gdir, exist_ok=True)
    import hashlib
    h = hashlib.sha256()
    for name in SHADERS:
        with open(os.path.join(shader_dir, name), "rb") as f:
            h.update(f.read())
    for name in ("ref_harness.cpp", "ref_harness_di.cpp", "ref_harness_post.cpp", "ref_common.h", "glsl_compat.h",
                 "alias_ref.cpp", "make_ref.py", "../detmath.h"):
        with open(os.path.join(HERE, name), "rb") as f:
            h.update(f.read())
    stamp = os.path.join(args.out, "stamp")
    outputs = [os.path.join(args.out, n) for n in ("libgrisref.so", "libdiref.so", "libpostref.so", "libaliasref.so")]
    if "--force" not in sys.argv and all(os.path.exists(o) for o in outputs) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read() == h.hexdigest():
                return 0
    for name in SHADERS:
        with open(os.path.join(shader_dir, name)) as f:
            src = f.read()
        with open(os.path.join(gdir, name), "w") as f:
            f.write(rewrite(name, src))
    so = os.path.join(args.out, "libgrisref.so")
    di = os.path.join(args.out, "libdiref.so")
    post = os.path.join(args.out, "libpostref.so")
    flags = [args.cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-fopenmp", "-Wl,-Bsymbolic",
             "-fsingle-precision-constant", "-ffp-contract=off", "-ftrivial-auto-var-init=zero",
             "-fno-strict-aliasing", "-Wno-unknown-pragmas", "-Wno-div-by-zero", "-I", gdir, "-I", HERE]
    for src, out in (("ref_harness.cpp", so), ("ref_harness_di.cpp", di), ("ref_harness_post.cpp", post)):
        r = subprocess.run(flags + [os.path.join(HERE, src), "-o", out])
        if r.returncode != 0:
            return r.returncode
    alias = os.path.join(args.out, "libaliasref.so")
    r = subprocess.run([args.cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I", os.path.join(args.reference, "src"), os.path.join(HERE, "alias_ref.cpp"), "-o", alias])
    if r.returncode != 0:
        return r.returncode
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    print(so)
    print(di)
    print(post)
    print(alias)
    return 0


if __name__ == "__main__":
    sys.exit(main())
