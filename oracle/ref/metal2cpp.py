"""Test infrastructure: mechanical rewrite of the reference's Metal shaders
(Sources/DenrimRendererKit/Resources/Shaders/PathTrace.metal, Denoise.metal)
into C++ that compiles against metal_shim.hpp.  The output is a build artefact written
only under oracle/_ref/; it is never committed and never hand-edited.

The rewrite changes no arithmetic.  It:
  1. drops the Metal headers and `using namespace` lines and every function
     that needs the hardware ray-tracing API (names containing `Hardware`),
     plus the compute kernels other than the requested ones (`pathTraceKernel`,
     `simpleSpatialDenoiseKernel`);
  2. strips `[[...]]` attributes;
  3. turns swizzle reads `.xyz/.xy/.xz` into calls and swizzle writes
     `v.xyz = e;` into `v.set_xyz(e);`;
  4. fixes the order of the random draws: where one statement draws more than
     once (`randomFloat(state)` in several arguments of one call), the draws
     are hoisted into temporaries in left-to-right textual order.  C++ leaves
     argument evaluation order unspecified (g++ evaluates right to left); the
     clang-based Metal compiler evaluates left to right.  A statement whose
     draws sit behind `&&`, `||` or `?:` is refused rather than reordered.
"""
import os
import re
import sys

HARDWARE = re.compile(r"\b\w*Hardware\w*\b|\braytracing\b|\bintersector\b|acceleration_structure")
DRAW = "randomFloat(state)"


def blank_comments(src: str) -> str:
    """Replaces comments by spaces (newlines kept) so offsets and lines survive."""
    out = []
    i, n = 0, len(src)
    while i < n:
        if src.startswith("//", i):
            j = src.find("\n", i)
            j = n if j < 0 else j
            out.append(" " * (j - i))
            i = j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2) + 2
            out.append(re.sub(r"[^\n]", " ", src[i:j]))
            i = j
        else:
            out.append(src[i])
            i += 1
    return "".join(out)


def top_level_items(src: str):
    """Yields (start, end, text) of top-level items: runs ending at a `;` or a
    closing brace at depth 0."""
    depth, start = 0, 0
    for i, ch in enumerate(src):
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth == 0:
                # a struct definition continues to its ';'
                j = i + 1
                while j < len(src) and src[j] in " \t\n":
                    j += 1
                if j < len(src) and src[j] == ";":
                    continue
                yield start, i + 1, src[start:i + 1]
                start = i + 1
        elif ch == ";" and depth == 0:
            yield start, i + 1, src[start:i + 1]
            start = i + 1
    yield start, len(src), src[start:]


def keep_item(text: str, kernels) -> bool:
    if HARDWARE.search(text):
        return False
    m = re.search(r"\bkernel\s+void\s+(\w+)", text)
    if m and m.group(1) not in kernels:
        return False
    return True


def statement_bounds(src: str, pos: int):
    """Start and end offsets of the statement containing `pos`."""
    depth = 0
    i = pos
    while i > 0:
        ch = src[i - 1]
        if ch in ")]":
            depth += 1
        elif ch in "([":
            if depth == 0:
                pass
            else:
                depth -= 1
        if depth == 0 and ch in ";{}":
            break
        i -= 1
    start = i
    depth = 0
    j = pos
    while j < len(src):
        ch = src[j]
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == ";" and depth <= 0:
            break
        j += 1
    return start, j + 1


def hoist_draws(src: str):
    report = []
    pos = 0
    out = []
    counter = 0
    done_until = 0
    while True:
        k = src.find(DRAW, pos)
        if k < 0:
            break
        s, e = statement_bounds(src, k)
        stmt = src[s:e]
        n = stmt.count(DRAW)
        if n < 2:
            pos = k + len(DRAW)
            continue
        head = stmt.strip()
        first = stmt.find(DRAW)
        guarded = stmt[:stmt.rfind(DRAW)]
        if re.match(r"(if|while|for|return|else)\b", head) or re.search(r"&&|\|\||\?", guarded[first:]):
            raise SystemExit(f"metal2cpp: refusing to reorder draws in: {head[:120]}")
        names = []
        body = stmt
        for _ in range(n):
            name = f"mref_draw{counter}"
            counter += 1
            names.append(name)
            body = body.replace(DRAW, name, 1)
        lead = re.match(r"\s*", stmt).group(0)
        hoisted = "".join(f"float {nm} = {DRAW}; " for nm in names)
        out.append(src[done_until:s])
        out.append(lead + hoisted + body.lstrip())
        report.append(" ".join(head.split())[:100])
        done_until = e
        pos = e
    out.append(src[done_until:])
    return "".join(out), report


def rewrite_swizzles(src: str) -> str:
    # writes: <lvalue>.xyz (op)= expr;
    pattern = re.compile(r"([A-Za-z_][\w\.\[\]]*)\.xyz\s*([-+*/]?)=(?!=)")
    pieces = []
    i = 0
    for m in pattern.finditer(src):
        if m.start() < i:
            continue
        lhs, op = m.group(1), m.group(2)
        depth, j = 0, m.end()
        while j < len(src):
            ch = src[j]
            if ch in "([":
                depth += 1
            elif ch in ")]":
                depth -= 1
            elif ch == ";" and depth == 0:
                break
            j += 1
        expr = src[m.end():j].strip()
        value = f"{lhs}.xyz {op} ({expr})" if op else f"({expr})"
        pieces.append(src[i:m.start()])
        pieces.append(f"{lhs}.set_xyz({value})")
        i = j
    pieces.append(src[i:])
    src = "".join(pieces)
    return re.sub(r"\.(xyz|xy|xz)\b(?!\s*\()", r".\1()", src)


def convert(metal_path: str, kernels=("pathTraceKernel",)) -> str:
    raw = open(metal_path).read()
    src = blank_comments(raw)
    src = re.sub(r"#include\s*<metal_\w+>", "", src)
    src = re.sub(r"using\s+namespace\s+(metal|raytracing)\s*;", "", src)
    items = [t for _, _, t in top_level_items(src) if keep_item(t, kernels)]
    src = "".join(items)
    src = re.sub(r"\[\[[^\]]*\]\]", "", src)
    src, hoisted = hoist_draws(src)
    src = rewrite_swizzles(src)
    header = (f"// Generated by oracle/ref/metal2cpp.py from the reference's {os.path.basename(metal_path)}.\n"
              "// Build artefact: do not edit, do not commit.\n"
              "#include \"metal_shim.hpp\"\nnamespace mref {\n")
    notes = "".join(f"// hoisted draws: {h}\n" for h in hoisted)
    footer = "\n}  // namespace mref\n#undef kernel\n#undef device\n#undef constant\n#undef thread\n#undef threadgroup\n"
    return header + notes + src + footer


if __name__ == "__main__":
    if len(sys.argv) < 3:
        raise SystemExit("usage: metal2cpp.py SHADER.metal out.cpp [kernel ...]")
    text = convert(sys.argv[1], tuple(sys.argv[3:]) or ("pathTraceKernel",))
    with open(sys.argv[2], "w") as f:
        f.write(text)
