"""Reader for tristan-ff input files (the `<block>` / `key = value # comment` format).

Follows parseInput / getInput of src/io/read_input.F90:56-102,138-384:
  * a block starts at a line whose first blank-delimited token is `<name>`;
  * only the first block of a given name is searched, up to the next line
    whose first token starts with `<`;
  * within it, the first line whose first token equals the key is taken; the
    value is the text between the first `=` and the first `#`, stripped;
  * a missing key takes the caller's default, and without a default it is an
    error (the reference calls throwError, read_input.F90:148-156).
"""
import os


class InputError(ValueError):
    pass


_MISSING = object()


class InputFile:
    def __init__(self, path):
        self.path = path
        if not os.path.exists(path):
            raise InputError("ERROR while reading input file: `%s`" % path)
        with open(path) as f:
            self.lines = f.read().splitlines()

    @staticmethod
    def _first_token(line):
        # list-directed read of a character variable: up to the first blank, comma or slash
        s = line.strip()
        for i, ch in enumerate(s):
            if ch in " \t,/":
                return s[:i]
        return s

    def raw(self, block, key):
        inside = False
        for line in self.lines:
            tok = self._first_token(line)
            if not inside:
                if tok == "<%s>" % block:
                    inside = True
                continue
            if tok.startswith("<"):
                return None
            if tok == key:
                k1 = line.find("=")
                k2 = line.find("#")
                if k2 < 0:
                    k2 = len(line)
                return line[k1 + 1:k2].strip()
        return None

    def get(self, block, key, typ=float, default=_MISSING):
        v = self.raw(block, key)
        if v is None or v == "":
            if default is _MISSING:
                raise InputError("ERROR: `%s` in block `%s` not found in the input file" % (key, block))
            return default
        if typ is int:
            return int(float(v)) if "." in v or "e" in v.lower() else int(v)
        if typ is float:
            return float(v.replace("d", "e").replace("D", "e"))
        return v


def read_input(path):
    return InputFile(path)


# <problem> keys of each shipped user file, in ffe_grid_desc.params order
PROBLEM_KEYS = {
    "psr": ("psr_radius", "psr_angle", "psr_period", "psr_bscale"),   # user/user_psr.F90:28-32
    "uniform": ("L0", "r_L0", "t0", "beta_twist"),                     # user/user_uniform.F90:29-32
    "loop": ("L0", "a_L0", "h_L0", "r_L0", "t0", "beta_twist"),        # user/user_loop.F90:29-34
    "none": (),
}
PROBLEM_DEFAULTS = {"psr_bscale": 1.0}


def desc_from_input(path, setup="none", precision="fp32", path_kind=0):
    """Build a GridDesc and the run settings from an input file.

    Returns (desc, settings) with settings = {"last": final_timestep,
    "output_start", "output_interval", "output_istep"}.
    """
    from . import make_desc, PRECISIONS, SETUPS  # local import: avoids a cycle
    f = read_input(path)
    size = tuple(f.get("grid", k, int) for k in ("mx0", "my0", "mz0"))
    bnd = [f.get("grid", k, int, 1) for k in ("boundary_x", "boundary_y", "boundary_z")]
    absorb = 20
    if 2 in bnd:                         # src/logistics/initialize.F90:144-148
        bnd = [2, 2, 2]
        absorb = f.get("grid", "absorb_buff", int, 20)
    cc = f.get("algorithm", "c", float, 0.45)
    params = [f.get("problem", k, float, PROBLEM_DEFAULTS.get(k, _MISSING)) for k in PROBLEM_KEYS[setup]]
    desc = make_desc(size, precision=PRECISIONS[precision], boundary=tuple(bnd), cc=cc,
                     absorb_buff=absorb, setup=SETUPS[setup], params=params, path=path_kind)
    settings = {
        "last": f.get("time", "last", int, 1000),
        "output_start": f.get("output", "start", int, 0),
        "output_interval": f.get("output", "interval", int, 10),
        "output_istep": f.get("output", "istep", int, 4),
    }
    return desc, settings
