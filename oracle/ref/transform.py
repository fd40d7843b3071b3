"""Mechanical OpenCL-C -> C++ text transform for Yune's kernel files.

TEST INFRASTRUCTURE: part of the recipe that compiles the reference kernels into
oracle/_ref/ (never committed). The transform changes syntax only, so the reference's
own arithmetic runs unchanged:
  * `#yune-preproc ...` header lines are dropped (src/CLManager.cpp:182-204 strips
    them the same way before clBuildProgram);
  * vector literals `(float4)(a, b, c, d)` / `(float4) x` become constructor calls
    (in C++ the cast form would be a comma expression);
  * address-space and access qualifiers (__kernel, __global, __constant, constant,
    __read_only, __write_only) are removed;
  * the `.xyz` swizzle becomes a call, `.xyz()`;
  * the tunable `#define`s (RR_THRESHOLD, LIGHT_SIZE, HEAP_SIZE, BDPT_BOUNCES) are
    wrapped in #ifndef so a variant can set them, and the GI loop bound 100000
    (udpt.cl:463) becomes YREF_MAX_DEPTH;
  * sampleLights gets an explicit `return -1;` where the reference falls off the end
    of a non-void function;
  * (variant B only, graft_oren_nayar below) udpt.cl's evaluateBRDF gets the Oren-Nayar
    diffuse rule of udpt-primitives.cl;
  * traverseBVH's candidate queue gets one spare entry: its loop checks the length only
    before a node's two children are pushed (udpt.cl:298,315-319, bdpt.cl likewise), so
    a full queue takes one write past its end, which the loop never reads. On the GPU
    that write goes unnoticed; compiled as C++ it would overwrite the stack.
Usage: python transform.py <in.cl> <out.inc>
"""
import re
import sys

TUNABLE = ("RR_THRESHOLD", "LIGHT_SIZE", "HEAP_SIZE", "BDPT_BOUNCES")


def transform(text: str) -> str:
    out = []
    for line in text.splitlines():
        if line.lstrip().startswith("#yune-preproc"):
            out.append("")
            continue
        m = re.match(r"\s*#define\s+(\w+)\s+(.*)$", line)
        if m and m.group(1) in TUNABLE:
            out.append(f"#ifndef {m.group(1)}\n#define {m.group(1)} {m.group(2).strip()}\n#endif")
            continue
        out.append(line)
    s = "\n".join(out) + "\n"
    # vector casts followed by a parenthesised list or a literal
    s = re.sub(r"\(\s*(float4|float3|int2)\s*\)\s*(?=\()", r"\1", s)
    s = re.sub(r"\(\s*(float4|float3|int2)\s*\)\s*([0-9][0-9.]*f?)", r"\1(\2)", s)
    for q in ("__kernel", "__global", "__constant", "__read_only", "__write_only"):
        s = re.sub(r"\b" + q + r"\b", "", s)
    s = re.sub(r"\bconstant\b", "", s)
    s = re.sub(r"\.xyz\b", ".xyz()", s)
    s = re.sub(r"i\s*<\s*100000\s*;", "i < YREF_MAX_DEPTH;", s)
    # sampleLights can run off its end (udpt.cl:681-698, bdpt.cl likewise); in C++ that
    # is undefined and the optimiser may assume it never happens, so give it the value
    # the restatement documents: -1, no light.
    s = re.sub(r"(cumulative_weight \+= weight;\s*\}\s*)\}", r"\1    return -1;\n}", s)
    s = re.sub(r"int\s+candidate_list\[HEAP_SIZE\]", "int candidate_list[HEAP_SIZE + 1]", s)
    return s


# ---- variant B: udpt.cl's evaluateBRDF with the Oren-Nayar rule of udpt-primitives.cl ----
# The benchmark configurations shade diffuse surfaces with Oren-Nayar, which Yune ships in
# kernels/legacy/udpt-primitives.cl (evaluateBRDF, :673-690, calling OrenNayarBRDF,
# :696-725, and the shading-frame helpers of :1147-1213) and not in udpt.cl. graft_oren_nayar
# builds that composite from the two files as they are: the helper functions and
# OrenNayarBRDF are taken verbatim (brace-matched), OrenNayarBRDF reads the material from
# udpt.cl's material buffer instead of the analytic scene's table (the two lines that
# differ are named below), and udpt.cl's diffuse branch calls it exactly where
# udpt-primitives.cl's does (rr_prob == 1). The glossy lobe keeps udpt.cl's exponent px + py.
ON_HELPERS = ("cosTheta", "cos2Theta", "sin2Theta", "sinTheta", "cosPhi", "sinPhi", "toShadingSpace",
              "OrenNayarBRDF")


def _function(text, name):
    """The full definition (return type to closing brace) of function `name`."""
    m = re.search(r"^[ \t]*(float4|float|int|bool)\s+" + name + r"\s*\([^;{]*\)\s*\{", text, re.M)
    if not m:
        raise ValueError("definition of %s not found" % name)
    depth, i = 0, m.end() - 1
    while True:
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():i + 1]
        i += 1


def graft_oren_nayar(udpt_text: str, prim_text: str) -> str:
    funcs = [_function(prim_text, n) for n in ON_HELPERS]
    on = funcs[-1]
    sig = re.match(r"[^(]*\(([^)]*)\)", on)
    on = on.replace(sig.group(0), "float4 OrenNayarBRDF(" + sig.group(1) + ", __global Material* mat_data)", 1)
    # the analytic scene's material lookup -> the triangle's material in udpt.cl's buffers
    on, n1 = re.subn(r"int\s+matID\s*=\s*getMatID\s*\(\s*hit_info\s*\)\s*;",
                     "int matID = scene_data[hit_info.triangle_ID].matID;", on)
    on, n2 = re.subn(r"\bmaterials\[", "mat_data[", on)
    if n1 != 1 or n2 < 1:
        raise ValueError("OrenNayarBRDF does not have the expected material lookup")
    on = on.replace("__global Material* mat_data)", "__global Triangle* scene_data, __global Material* mat_data)", 1)
    funcs[-1] = on
    block = "\n\n".join(funcs) + "\n\n"
    m = re.search(r"^float4\s+evaluateBRDF\s*\([^;{]*\)\s*\{", udpt_text, re.M)
    if not m:
        raise ValueError("evaluateBRDF definition not found in udpt.cl")
    body_start = m.start()
    diffuse = re.compile(r"if\s*\(\s*!sample_glossy\s*\)\s*\n(\s*)color\s*=\s*(mat_data\[matID\]\.kd\s*\*\s*INV_PI\s*/\s*rr_prob)\s*;")
    tail = udpt_text[body_start:]
    d = diffuse.search(tail)
    if not d:
        raise ValueError("udpt.cl's diffuse branch not found")
    ind = d.group(1)
    repl = ("if(!sample_glossy)\n" + ind + "{\n" + ind + "    if(rr_prob == 1.0f)\n" + ind +
            "        color = OrenNayarBRDF(w_i, w_o, hit_info, scene_data, mat_data);\n" + ind + "    else\n" + ind +
            "        color = " + d.group(2) + ";\n" + ind + "}")
    tail = tail[:d.start()] + repl + tail[d.end():]
    return udpt_text[:body_start] + block + tail


def main(argv):
    src, dst = argv[1], argv[2]
    with open(src, "r", encoding="utf-8", errors="replace") as f:
        text = f.read()
    with open(dst, "w") as f:
        f.write(transform(text))


if __name__ == "__main__":
    main(sys.argv)
