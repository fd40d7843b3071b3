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


def main(argv):
    src, dst = argv[1], argv[2]
    with open(src, "r", encoding="utf-8", errors="replace") as f:
        text = f.read()
    with open(dst, "w") as f:
        f.write(transform(text))


if __name__ == "__main__":
    main(sys.argv)
