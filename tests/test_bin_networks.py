"""The in-bucket sorting networks of k_bin_fix (fl_bin.cu) sort every input.

By the 0-1 principle a comparator network sorts every input iff it sorts every
sequence of 0s and 1s; the test reads the comparators from the kernel source
and applies them to all 2^8 / 2^16 binary inputs at once."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "fluid-simulation_gb300", "csrc", "fl_bin.cu")


def network(name):
    src = open(SRC).read()
    body = re.search(r"void %s\(uint32_t \(&a\)\[16\]\) \{(.*?)\n\}" % name, src, re.S).group(1)
    return [(int(i), int(j)) for i, j in re.findall(r"BIN_CX\((\d+), (\d+)\)", body)]


def sorts_all_binary_inputs(net, n):
    x = ((np.arange(1 << n)[:, None] >> np.arange(n)[None, :]) & 1).astype(np.uint8)
    for i, j in net:
        lo = np.minimum(x[:, i], x[:, j])
        hi = np.maximum(x[:, i], x[:, j])
        x[:, i], x[:, j] = lo, hi
    return bool(np.all(x[:, :-1] <= x[:, 1:]))


def test_sort8_network():
    net = network("sort8")
    assert len(net) == 19 and all(i < j < 8 for i, j in net)
    assert sorts_all_binary_inputs(net, 8)


def test_sort16_network():
    net = network("sort16")
    assert len(net) == 63 and all(i < j < 16 for i, j in net)
    assert sorts_all_binary_inputs(net, 16)
