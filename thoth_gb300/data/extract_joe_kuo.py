"""Extract the Joe-Kuo "new-joe-kuo-6.21201" direction-number dataset.

The dataset (S. Joe and F. Y. Kuo, https://web.maths.unsw.edu.au/~fkuo/sobol/)
is published data; the reference embeds its first 4096 file dimensions as C
arrays in pricer/src/nodes/sobol_direction_numbers.cpp:16-70004 (S = degrees,
A = packed polynomial coefficients, M_OFFSET/M = initial direction numbers).
Bit-exact Sobol parity requires the same table, so this script parses that
file once and writes the compact binary joe_kuo_6_21201.bin next to it:

    magic   8 bytes  b"JK621201"
    dims    uint32   number of file dimensions (4096)
    nm      uint32   number of m values
    S       uint32[dims]
    A       uint32[dims]
    MOFF    uint32[dims + 1]
    M       uint32[nm]

All integers little-endian. Usage: python extract_joe_kuo.py [reference root]
(default: $THOTH_REFERENCE).
"""
import os
import pathlib
import re
import struct
import sys


def parse_array(text, name):
    m = re.search(r"sobol_jk::%s\[\d+\]\s*=\s*\{(.*?)\};" % name, text, re.S)
    if not m:
        raise SystemExit("array %s not found" % name)
    return [int(v) for v in re.findall(r"\d+", m.group(1))]


def main():
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("THOTH_REFERENCE")
    if not arg:
        raise SystemExit("usage: extract_joe_kuo.py <reference root> (or set THOTH_REFERENCE)")
    root = pathlib.Path(arg)
    src = (root / "pricer/src/nodes/sobol_direction_numbers.cpp").read_text()
    dims = int(re.search(r"FILE_DIMS\s*=\s*(\d+)", src).group(1))
    S = parse_array(src, "S")
    A = parse_array(src, "A")
    MOFF = parse_array(src, "M_OFFSET")
    M = parse_array(src, "M")
    assert len(S) == dims and len(A) == dims and len(MOFF) == dims + 1 and MOFF[-1] == len(M)
    out = pathlib.Path(__file__).with_name("joe_kuo_6_21201.bin")
    with open(out, "wb") as f:
        f.write(b"JK621201")
        f.write(struct.pack("<II", dims, len(M)))
        for arr in (S, A, MOFF, M):
            f.write(struct.pack("<%dI" % len(arr), *arr))
    print("wrote", out, dims, "dims", len(M), "m values")


if __name__ == "__main__":
    main()
