"""The .conf section reader against the reference's own reader on seeded
random files (CPU).

The reference's reader (src/config.c:19-106) cuts the file with the C
library's tokenizer, so malformed files (text before the first `$`, empty
titles, sections without text, `$` inside titles or mid-line, more than
eight sections, a second load without an unload) split in ways a plain
reading of the format does not predict.  Files are drawn from fragments
that hit those cases; both readers load each file, and every title any
`$` could start (and a few that no file holds) must give the same section
text, or no section, in both.

Runs where oracle/_ref/libref_psdata.so was built from the reference's
sources; skipped elsewhere.
"""
import ctypes

import numpy as np
import pytest

from oracle import ref
from sph import bindings as bnd

pytestmark = pytest.mark.skipif(not ref.available("psdata"), reason="reference reader not built")

N_FILES = 1500
TITLES = ["psdata_specification", "opencl_kernel_files", "a", "b c", " a", "a "]
BODIES = ["pnum | 1 | unsigned int | 8\n", "common, fluids\n", "# c\n", "x\n", "\n", " ", "k | 3 | float\n"]
NOISE = ["$", "$$", "\n", "\n\n", "$\n", "text", " ", "|", "a$b"]


def random_conf(rng):
    parts = []
    if rng.integers(3) == 0:
        parts.append(NOISE[int(rng.integers(len(NOISE)))] + "lead\n")  # text before the first section
    for _ in range(int(rng.integers(0, 11))):
        form = rng.integers(10)
        if form < 6:
            # a well-formed section
            parts.append("$" + TITLES[int(rng.integers(len(TITLES)))] + "\n")
            parts.extend(BODIES[int(rng.integers(len(BODIES)))] for _ in range(int(rng.integers(0, 3))))
        elif form < 8:
            parts.append(NOISE[int(rng.integers(len(NOISE)))])
        else:
            parts.append("$" + TITLES[int(rng.integers(len(TITLES)))])  # a title without its newline
    text = "".join(parts)
    if text and rng.integers(4) == 0:
        text = text.rstrip("\n")
    return text.encode()


def candidate_titles(data):
    """Every string a title could be: the run after each `$` up to the end
    of its line (raw and with leading newlines skipped), the names used,
    and names no file holds."""
    names = {t.encode() for t in TITLES} | {b"", b"nosuch", b"lead"}
    for i, c in enumerate(data):
        if c == ord("$"):
            rest = data[i + 1:]
            names.add(rest.split(b"\n", 1)[0])
            stripped = rest.lstrip(b"\n")
            names.add(stripped.split(b"\n", 1)[0])
            if rest[:1] == b"\n":
                # a `$` at the start of the file keeps the newlines after it
                cut = len(rest) - len(stripped)
                names.add(rest[:cut] + stripped.split(b"\n", 1)[0])
    return sorted(names)


def reference_reader():
    lib = ref.psdata_lib()
    lib.load_config.argtypes = [ctypes.c_char_p]
    lib.load_config.restype = ctypes.c_int
    lib.get_config_section.argtypes = [ctypes.c_char_p]
    lib.get_config_section.restype = ctypes.c_char_p
    lib.unload_config.argtypes = []
    lib.unload_config.restype = None
    return lib


def test_reader_equals_reference_reader_on_random_files(tmp_path):
    lib = reference_reader()
    rng = np.random.default_rng(7)
    for case in range(N_FILES):
        files = [random_conf(rng) for _ in range(2 if rng.integers(5) == 0 else 1)]
        names = set()
        for k, data in enumerate(files):
            path = tmp_path / ("c%d.conf" % k)
            path.write_bytes(data)
            assert lib.load_config(str(path).encode()) == 0
            assert bnd.load_config(str(path)) == 0
            names.update(candidate_titles(data))
        try:
            for name in sorted(names):
                assert bnd.get_config_section(name) == lib.get_config_section(name), (files, name)
        finally:
            lib.unload_config()
            bnd.unload_config()


def test_missing_file_is_reported_by_both(tmp_path):
    lib = reference_reader()
    path = str(tmp_path / "absent.conf")
    assert lib.load_config(path.encode()) == 1
    assert bnd.load_config(path) == 1
