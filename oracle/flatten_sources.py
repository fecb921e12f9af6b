"""Writes one C++ translation unit with the project headers of a source inlined.

Used by oracle/build_ref.sh: the test driver of include/pasc/gb300_backend.hpp runs the
reference's own generic solver templates, whose headers exist only where the reference tree
is.  The recipe inlines every quoted include found under the given directories (each file
once; the reference's headers carry include guards) and keeps system includes and includes it
cannot resolve (this repository's own headers), so that the output compiles on a machine that
has this repository but not the reference tree.  The output is a build product: it goes to
oracle/_ref/ only.

  python flatten_sources.py OUT ENTRY [ENTRY ...] -I DIR [-I DIR ...]
"""
from __future__ import annotations

import os
import re
import sys

INC = re.compile(r'^\s*#\s*include\s+"([^"]+)"')


def flatten(path, dirs, done, out):
    path = os.path.realpath(path)
    if path in done:
        return
    done.add(path)
    here = os.path.dirname(path)
    with open(path, errors="replace") as f:
        for line in f:
            m = INC.match(line)
            if m:
                name = m.group(1)
                for d in [here] + dirs:
                    cand = os.path.join(d, name)
                    if os.path.isfile(cand) and any(os.path.realpath(cand).startswith(os.path.realpath(x) + os.sep)
                                                    for x in dirs):
                        flatten(cand, dirs, done, out)
                        break
                else:
                    out.append(line)
                continue
            out.append(line)
    out.append("\n")


def main(argv):
    out_path, rest = argv[0], argv[1:]
    entries, dirs = [], []
    i = 0
    while i < len(rest):
        if rest[i] == "-I":
            dirs.append(rest[i + 1])
            i += 2
        else:
            entries.append(rest[i])
            i += 1
    out, done = [], set()
    for e in entries:
        flatten(e, dirs, done, out)
    os.makedirs(os.path.dirname(out_path), exist_ok=True)
    with open(out_path, "w") as f:
        f.writelines(out)


if __name__ == "__main__":
    main(sys.argv[1:])
