"""Regenerate the SPIR-V decoder golden vectors from the reference's own tests.

The reference pins its SPIR-V decoder with three binary modules (spirv-parser/test_inputs/test.spv,
test2.spv, test3.spv) and the exact dump text each must produce (raw strings in
spirv-parser/src/lib.rs, tests parse_test, parse_test2, parse_test3).  This script copies the
modules and extracts the expected text into tests/golden/spirv/ so that the tests run without the
reference checkout.  Usage: python tests/golden/make_spirv_golden.py REFERENCE_ROOT (the checkout of
kazan-3d/kazan to read the modules and dumps from)
"""
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    src = os.path.join(ref_root, "spirv-parser")
    out = os.path.join(HERE, "spirv")
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(src, "src", "lib.rs"), encoding="utf-8") as f:
        text = f.read()
    # each test: include_bytes!("../test_inputs/NAME.spv") ... let expected = r#"...."#;
    pattern = re.compile(r'include_bytes!\("\.\./test_inputs/(\w+)\.spv"\).*?let expected = r#"(.*?)"#;', re.S)
    found = 0
    for name, expected in pattern.findall(text):
        shutil.copyfile(os.path.join(src, "test_inputs", name + ".spv"), os.path.join(out, name + ".spv"))
        with open(os.path.join(out, name + ".dis"), "w", encoding="utf-8") as f:
            f.write(expected)
        found += 1
    print("wrote %d golden modules to %s" % (found, out))
    return 0 if found == 3 else 1


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_spirv_golden.py REFERENCE_ROOT")
    sys.exit(main(sys.argv[1]))
