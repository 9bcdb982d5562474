"""numpy mirrors of the reference's FDPS particle / force classes.

Each dtype reproduces the byte layout of the C struct of the same name in
``include/sph_gb300.h`` (and therefore of the reference class it mirrors), so a
structured array can be handed to the C ABI as a plain pointer.

Reference classes (yamauchi1132/Research_Codes, sph_yamauchi/run):
  DensityEPI  hdr_density.hpp:33-58     DensityEPJ hdr_density.hpp:60-78
  Density     hdr_density.hpp:4-22
  HydroEPI    hdr_hydro.hpp:28-75       HydroEPJ   hdr_hydro.hpp:77-126
  Hydro       hdr_hydro.hpp:3-17
  GravityEPI  hdr_gravity.hpp:130-155   GravityEPJ hdr_gravity.hpp:157-192
  GravitySPJ  hdr_gravity.hpp:63-91     Gravity    hdr_gravity.hpp:95-105
"""
import numpy as np

_V3 = (np.float64, (3,))

DensityEPI = np.dtype([("id", np.int32), ("mass", np.float64), ("pos", _V3), ("vel", _V3),
                       ("ksr", np.float64), ("rs", np.float64)], align=True)
DensityEPJ = np.dtype([("id", np.int32), ("mass", np.float64), ("pos", _V3), ("vel", _V3)],
                      align=True)
Density = np.dtype([("dens", np.float64), ("divv", np.float64), ("rotv", np.float64),
                    ("grdh", np.float64), ("ksr", np.float64), ("np", np.int64),
                    ("itr", np.bool_)], align=True)

_HYDRO_TAIL = [("ksr", np.float64), ("hinv", np.float64), ("pres", np.float64),
               ("presc", np.float64), ("bswt", np.float64), ("dens", np.float64),
               ("vsnd", np.float64), ("alph", np.float64), ("alphu", np.float64),
               ("thrm", np.float64), ("eta", np.float64)]
HydroEPI = np.dtype([("id", np.int64), ("pos", _V3), ("vel", _V3)] + _HYDRO_TAIL, align=True)
HydroEPJ = np.dtype([("id", np.int64), ("mass", np.float64), ("pos", _V3), ("vel", _V3)]
                    + _HYDRO_TAIL, align=True)
Hydro = np.dtype([("acch", _V3), ("accg", _V3), ("udot", np.float64), ("vsmx", np.float64),
                  ("diffu", np.float64)], align=True)

GravityEPI = np.dtype([("pos", _V3), ("eps2", np.float64)], align=True)
GravityEPJ = np.dtype([("mass", np.float64), ("pos", _V3), ("eps2", np.float64)], align=True)
GravitySPJ = np.dtype([("mass", np.float64), ("pos", _V3), ("eps2", np.float64)], align=True)
Gravity = np.dtype([("acc", _V3), ("pot", np.float64), ("eta", np.float64)], align=True)

# Order used by sph_abi_layout().
LAYOUT_ORDER = [("DensityEPI", DensityEPI), ("DensityEPJ", DensityEPJ), ("Density", Density),
                ("HydroEPI", HydroEPI), ("HydroEPJ", HydroEPJ), ("Hydro", Hydro),
                ("GravityEPI", GravityEPI), ("GravityEPJ", GravityEPJ),
                ("GravitySPJ", GravitySPJ), ("Gravity", Gravity)]

EXPECTED_SIZES = {"DensityEPI": 80, "DensityEPJ": 64, "Density": 56, "HydroEPI": 144,
                  "HydroEPJ": 152, "Hydro": 72, "GravityEPI": 32, "GravityEPJ": 40,
                  "GravitySPJ": 40, "Gravity": 40}


def layout_vector():
    """sizeof + field offsets in declaration order, as sph_abi_layout() reports."""
    out = []
    for _, dt in LAYOUT_ORDER:
        out.append(dt.itemsize)
        for name in dt.names:
            out.append(dt.fields[name][1])
    return out


# Status codes (enum sph_status).
SPH_OK = 0
SPH_ERR_INVALID_ARGUMENT = 1
SPH_ERR_CAPACITY = 2
SPH_ERR_CUDA = 3
SPH_ERR_NONFINITE = 4
SPH_ERR_NOT_CONVERGED = 5
SPH_ERR_STATE = 6
SPH_ERR_NO_DEVICE = 7

STATUS_NAMES = {0: "SPH_OK", 1: "SPH_ERR_INVALID_ARGUMENT", 2: "SPH_ERR_CAPACITY",
                3: "SPH_ERR_CUDA", 4: "SPH_ERR_NONFINITE", 5: "SPH_ERR_NOT_CONVERGED",
                6: "SPH_ERR_STATE", 7: "SPH_ERR_NO_DEVICE"}

# enum sph_precision
PREC_FP32C = 0
PREC_FP64 = 1


class SPHError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, status, detail=""):
        self.status = status
        name = STATUS_NAMES.get(status, f"status {status}")
        super().__init__(f"{name}: {detail}" if detail else name)
