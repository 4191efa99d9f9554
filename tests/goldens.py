"""Load the committed golden fixtures (tests/golden/*.npz) into ABI inputs."""
import json
import os

import numpy as np

from qlens_gb300 import abi

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["tiny_sie", "fixed_grid", "powerlaw", "nfw", "twoplane", "cfg1", "fits_synth", "hst_fits",
         "cfg2_draw", "cfg5_m200"]
# cases at the benchmarked workloads' sizes (slimmed fixtures, see Golden.exact)
LARGE_CASES = ["cfg2_draw", "cfg5_m200"]
REGOPT_CASES = ["regopt_tiny_sie", "regopt_powerlaw"]


class Golden:
    def __init__(self, name):
        self.name = name
        z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        self.arr = {k: z[k] for k in z.files}
        self.meta = json.loads(bytes(self.arr.pop("meta_json")).decode())
        self.sc = self.meta["scalars"]
        self.lenses = self.meta["lenses"]
        self.slim = self.meta.get("slim")
        if "L_index" in self.arr:
            self.arr["L_index"] = self.arr["L_index"].astype(np.int32)
        nx, ny = int(self.sc["nx"]), int(self.sc["ny"])
        self.nx, self.ny = nx, ny
        covinv = self.arr["covinv"] if int(self.sc["use_noise_map"]) else None
        self.image = abi.ImageBuffers(self.arr["xvals"], self.arr["yvals"], self.arr["data"],
                                      self.arr["mask"], covinv, self.sc["background_pixel_noise"])
        psf = self.arr["psf"].reshape(int(self.sc["psf_nx"]), int(self.sc["psf_ny"]))
        self.psf = abi.PSFBuffer(psf)
        o = abi.srcgrid_defaults()
        o.nsplit = int(self.sc["nsplit"])
        o.npixels_x = int(self.sc["srcgrid_nx"])
        o.npixels_y = int(self.sc["srcgrid_ny"])
        o.regparam = float(self.sc["regparam"])
        o.regularization = 1
        o.auto_sourcegrid = 1
        for line in self.meta["script"].splitlines():
            w = line.split()
            if w and w[0] == "srcgrid" and len(w) == 5:
                o.auto_sourcegrid = 0
                o.xmin, o.xmax, o.ymin, o.ymax = map(float, w[1:])
        self.opts = o

    @property
    def n_sub(self):
        """Sub-pixels (ray-traced points) of the masked pixels."""
        return int(self.arr["masked_pixels"].size) * int(self.sc["nsplit"]) ** 2

    def exact(self, name, a):
        """Bit-for-bit equality of an array with the reference's: by value, or
        for the slimmed arrays of the large cases by SHA-256 of the bytes."""
        if self.slim and name in self.slim["sha256"]:
            import hashlib
            ref_dtype = np.float64
            b = np.ascontiguousarray(np.asarray(a, dtype=ref_dtype)).tobytes()
            return hashlib.sha256(b).hexdigest() == self.slim["sha256"][name]
        return np.array_equal(a, self.arr[name])

    def sample(self, name, a=None):
        """(reference values, the same elements of a): everything, or every
        stride-th element for the slimmed arrays of the large cases."""
        if self.slim and name in self.slim["sha256"]:
            ref = self.arr[name + "_sub"]
            return ref, (None if a is None else np.asarray(a)[::self.slim["stride"]])
        return self.arr[name], a

    @property
    def regopt(self):
        """(minlog, maxlog, tol, max_iter) of QLens's 'optimize_regparam on'
        (its defaults, lens.cpp:421-425) when the case was run with it, else None."""
        return (-3.0, 5.0, 0.01, 20) if int(self.sc.get("regopt", 0)) else None

    def params(self):
        return abi.flat_params(self.lenses)

    def zbeta(self):
        """(zfactors, betafactors rows) the reference ray-traced this case with,
        or (None, None) for a single lens plane."""
        zf = self.arr.get("zfactors")
        if zf is None or len(zf) <= 1:
            return None, None
        bf = list(self.arr["betafactors"])
        beta, k = [], 0
        for i in range(1, len(zf)):
            beta.append(bf[k:k + i])
            k += i
        return list(zf), beta

    def planes(self):
        return abi.make_planes(*self.zbeta())
