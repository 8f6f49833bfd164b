"""Every reference check that the engine and the oracle report as "Assertion failed (file:line):
condition" cites the line of the reference's sources that holds that condition (a wrong line is a
message the reference never prints).  Runs where the reference's sources are present (the build
container); skipped elsewhere."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_dir():
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    return g.REFERENCE_DIR


def _unescape(s):
    return s.replace('\\"', '"').replace("\\\\", "\\")


def _cited_messages():
    """(source file of the message, cited file, cited line, condition) of every such message."""
    out = []
    net = open(os.path.join(ROOT, "spice2_gb300", "csrc", "net.cu")).read()
    for m in re.finditer(r'pre_failed\("([\w.]+):(\d+)",\s*"((?:[^"\\]|\\.)*)"\)', net):
        out.append(("net.cu", m.group(1), int(m.group(2)), _unescape(m.group(3))))
    ora = open(os.path.join(ROOT, "oracle", "spice_oracle.c")).read()
    for m in re.finditer(r'"Assertion failed \(([\w.]+):(\d+)\): ((?:[^"\\]|\\.)*)"', ora):
        out.append(("spice_oracle.c", m.group(1), int(m.group(2)), _unescape(m.group(3))))
    return out


def test_messages_are_found():
    msgs = _cited_messages()
    assert sum(1 for m in msgs if m[0] == "net.cu") >= 10 and sum(1 for m in msgs if m[0] == "spice_oracle.c") >= 10


@pytest.mark.skipif(not os.path.isdir(os.path.join(_reference_dir(), "spice")), reason="reference sources not present")
def test_cited_lines_hold_the_conditions():
    files = {}
    for dirpath, _, names in os.walk(os.path.join(_reference_dir(), "spice")):
        for name in names:
            files.setdefault(name, os.path.join(dirpath, name))
    squash = lambda t: re.sub(r"\s+", "", t)
    bad = []
    for where, name, line, cond in _cited_messages():
        lines = open(files[name]).read().splitlines()
        window = "".join(lines[line - 1:line + 2])  # a check may continue over the next lines
        if "SPICE_" not in lines[line - 1] or squash(cond) not in squash(window):
            bad.append(f"{where}: {name}:{line} does not hold {cond!r}")
    assert not bad, "\n".join(bad)
