"""Minimal pure-Python stand-in for the ``bitarray`` package.

Test infrastructure only: it lets the reference implementation (which imports
``bitarray``) run in this container so that ``make_golden.py`` can record its
outputs as fixtures.  Only the subset the reference uses is provided:
construction from a '0'/'1' string or a length, ``frombytes``/``tobytes``
(MSB-first, zero padded to whole bytes), item/slice access, ``count``,
``copy``, ``to01``, ``__eq__`` and ``__len__``.
"""


class bitarray:
    __slots__ = ("_b",)

    def __init__(self, init=0):
        if isinstance(init, str):
            self._b = [1 if ch == "1" else 0 for ch in init if ch in "01"]
        elif isinstance(init, int):
            self._b = [0] * init
        elif isinstance(init, (list, tuple)):
            self._b = [1 if x else 0 for x in init]
        else:
            raise TypeError("unsupported bitarray initialiser")

    def frombytes(self, data):
        for byte in data:
            for k in range(7, -1, -1):
                self._b.append((byte >> k) & 1)

    def tobytes(self):
        bits = self._b + [0] * ((-len(self._b)) % 8)
        out = bytearray()
        for k in range(0, len(bits), 8):
            v = 0
            for bit in bits[k : k + 8]:
                v = (v << 1) | bit
            out.append(v)
        return bytes(out)

    def __getitem__(self, key):
        if isinstance(key, slice):
            new = bitarray(0)
            new._b = self._b[key]
            return new
        return bool(self._b[key])

    def __setitem__(self, key, value):
        self._b[key] = 1 if value else 0

    def count(self, value=1):
        s = sum(self._b)
        return s if value else len(self._b) - s

    def copy(self):
        new = bitarray(0)
        new._b = list(self._b)
        return new

    def to01(self):
        return "".join("1" if x else "0" for x in self._b)

    def __eq__(self, other):
        return isinstance(other, bitarray) and self._b == other._b

    def __len__(self):
        return len(self._b)

    def __repr__(self):
        return "bitarray('%s')" % self.to01()
