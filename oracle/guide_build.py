"""TEST INFRASTRUCTURE ONLY: prepares the integration guide's C++ for `make ref`.

    python oracle/guide_build.py <reference src folder> <output folder>

Writes into the output folder (oracle/_ref, never committed):
  patched/cgs.hpp     the reference's src/cgs.hpp with the four one-line
                      accessors INTEGRATION.md section 2 asks a maintainer to
                      add (object::get_trans_mat, object::get_invert,
                      cylinder::get_r1_sq, cylinder::get_r2_sq), inserted after
                      the members they sit beside;
  guide_flatten.inc   the C++ block of INTEGRATION.md section 2, verbatim.
ref_shim.cpp includes the second and is compiled against the first, so the
golden CSG programs come from the guide's own walk.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
GUIDE = os.path.join(HERE, "..", "INTEGRATION.md")

ACCESSORS = [
    ("    void set_trans_mat(const mat3x3& new_mat) { trans_mat = new_mat; }\n",
     "    const mat3x3& get_trans_mat() const { return trans_mat; }\n"
     "    int get_invert() const { return invert; }\n"),
    ("    double get_r2() const { return sqrt(r2_sq); }\n",
     "    double get_r1_sq() const { return r1_sq; }\n"
     "    double get_r2_sq() const { return r2_sq; }\n"),
]


def patched_header(src):
    text = open(os.path.join(src, "cgs.hpp")).read()
    for anchor, add in ACCESSORS:
        if text.count(anchor) != 1:
            raise SystemExit(f"cgs.hpp: anchor not found once: {anchor.strip()}")
        text = text.replace(anchor, anchor + add)
    return text


def guide_block():
    md = open(GUIDE).read()
    sec = md[md.index("## 2. "):md.index("## 3. ")]
    blocks = re.findall(r"```cpp\n(.*?)```", sec, re.S)
    if len(blocks) != 1:
        raise SystemExit("INTEGRATION.md section 2 must hold exactly one C++ block")
    return blocks[0]


def main(src, out):
    os.makedirs(os.path.join(out, "patched"), exist_ok=True)
    with open(os.path.join(out, "patched", "cgs.hpp"), "w") as fh:
        fh.write(patched_header(src))
    with open(os.path.join(out, "guide_flatten.inc"), "w") as fh:
        fh.write("// generated from INTEGRATION.md section 2 by oracle/guide_build.py\n" + guide_block())


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
