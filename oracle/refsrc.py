"""Where the lyspeq source tree is (test infrastructure).

The oracle compiles lyspeq's own translation units and reads its test
fixtures from that tree.  Its location is the environment variable
LYSPEQ_SRC; without it, the default that the build recipe
(oracle/refbuild/Makefile, `LYSPEQ_SRC ?= ...`) names.  The tree exists only
on the machine that generates fixtures; every caller treats its absence as
"skip".
"""
from __future__ import annotations

import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root() -> str:
    env = os.environ.get("LYSPEQ_SRC")
    if env:
        return env
    with open(os.path.join(HERE, "refbuild", "Makefile")) as f:
        for line in f:
            m = re.match(r"\s*LYSPEQ_SRC\s*\?=\s*(\S+)", line)
            if m:
                return m.group(1)
    return ""
