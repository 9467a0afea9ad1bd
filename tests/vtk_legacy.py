"""Minimal reader of legacy VTK files with BINARY (big-endian) payloads, for
checking the run-directory files: header lines, STRUCTURED_POINTS /
STRUCTURED_GRID geometry, FIELD arrays, POINTS, and POINT_DATA VECTORS /
SCALARS (with their LOOKUP_TABLE line), as the legacy-format readers the
reference's python/glemur/data.py uses (vtkStructuredPointsReader,
vtkStructuredGridReader) parse them."""
import numpy as np

_TYPES = {"float": ">f4", "double": ">f8", "int": ">i4"}


class LegacyVtk:
    def __init__(self, path):
        self.raw = open(path, "rb").read()
        self.pos = 0
        self.header = [self._line() for _ in range(4)]
        assert self.header[0] == "# vtk DataFile Version 2.0"
        assert self.header[2] == "BINARY"
        self.dataset = self.header[3].split()[1]
        self.field = {}
        self.point_data = {}
        self.points = None
        self.lines = list(self.header)
        while self.pos < len(self.raw):
            ln = self._line()
            self.lines.append(ln)
            tok = ln.split()
            key = tok[0]
            if key == "DIMENSIONS":
                self.dims = tuple(int(v) for v in tok[1:4])
            elif key in ("ORIGIN", "SPACING"):
                setattr(self, key.lower(), tuple(float(v) for v in tok[1:4]))
            elif key == "FIELD":
                for _ in range(int(tok[2])):
                    fl = self._line()
                    self.lines.append(fl)
                    name, nc, nt, ty = fl.split()
                    self.field[name] = self._array(ty, int(nc) * int(nt))
            elif key == "POINTS":
                self.points = self._array(tok[2], 3 * int(tok[1])).reshape(-1, 3)
            elif key == "POINT_DATA":
                self.npoints = int(tok[1])
            elif key == "VECTORS":
                self.point_data[tok[1]] = self._array(tok[2], 3 * self.npoints).reshape(-1, 3)
            elif key == "SCALARS":
                lt = self._line()
                self.lines.append(lt)
                assert lt == "LOOKUP_TABLE default", lt
                self.point_data[tok[1]] = self._array(tok[2], self.npoints)
            else:
                raise ValueError(f"unexpected line {ln!r}")

    def _line(self):
        e = self.raw.index(b"\n", self.pos)
        s = self.raw[self.pos:e].decode("ascii")
        self.pos = e + 1
        return s

    def _array(self, ty, n):
        dt = np.dtype(_TYPES[ty])
        a = np.frombuffer(self.raw, dtype=dt, count=n, offset=self.pos)
        self.pos += n * dt.itemsize
        return a.astype(dt.newbyteorder("="))
