"""Extract the reference's built-in benchmark inputs (JSON text held in
src/mcx_bench.h, the inputs of `mcxcl --bench <name>`) into
tests/golden/bench_<name>.json, so the JSON reader is tested on the
reference's own input files without the reference present.

    python tests/golden/make_json_fixtures.py --reference <reference checkout>

The colin27 entry is left out: its volume is an atlas embedded as encoded
binary data, outside the reader's scope.
"""
import argparse
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MCX_REFERENCE"),
                    help="the reference checkout (default: $MCX_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        sys.exit("name the reference checkout with --reference or MCX_REFERENCE")
    text = open(os.path.join(args.reference, "src", "mcx_bench.h")).read()
    names = re.search(r"benchname\[\]\s*=\s*\{([^}]*)\}", text).group(1)
    names = [n for n in re.findall(r'"([^"]*)"', names) if n]
    body = text[text.index("benchjson[]"):]
    entries = []
    pos = 0
    while True:
        k = body.find("MSTR(", pos)
        if k < 0:
            break
        depth, i = 0, k + 4
        while True:                      # the macro argument: balanced parentheses
            c = body[i]
            depth += (c == "(") - (c == ")")
            i += 1
            if depth == 0:
                break
        entries.append(body[k + 5:i - 1])
        pos = i
    for name, js in zip(names, entries):
        if name == "colin27":
            continue
        obj = json.loads(js)             # checks the extraction
        with open(os.path.join(HERE, "bench_%s.json" % name), "w") as f:
            json.dump(obj, f, indent=1)
            f.write("\n")
        print(name, len(js))


if __name__ == "__main__":
    main()
