"""Code units of the reference (hdr_heos.hpp:53-104).

L = 1e-3 R_sun, M = 1e-6 M_sun, T = 1 s; G expressed in those units.
"""
SOLAR_RADIUS = 6.9599e10      # cm   (hdr_heos.hpp:54)
SOLAR_MASS = 1.9891e33        # g    (hdr_heos.hpp:55)
GRAVITY_CGS = 6.6738480e-8    # cgs  (hdr_heos.hpp:56)

UNIT_LENGTH = SOLAR_RADIUS * 1.0e-3   # hdr_heos.hpp:67
UNIT_MASS = SOLAR_MASS * 1.0e-6       # hdr_heos.hpp:68
UNIT_TIME = 1.0                       # hdr_heos.hpp:69
UNIT_VELOCITY = UNIT_LENGTH / UNIT_TIME
UNIT_DENSITY = UNIT_MASS / UNIT_LENGTH ** 3
UNIT_ENERGY = UNIT_VELOCITY ** 2      # specific energy
UNIT_PRESSURE = UNIT_MASS / (UNIT_LENGTH * UNIT_TIME ** 2)
UNIT_ACCELERATION = UNIT_VELOCITY / UNIT_TIME

# GravityConstantInThisUnit, hdr_heos.hpp:102-104
G = GRAVITY_CGS / (UNIT_LENGTH ** 3 / UNIT_MASS / UNIT_TIME ** 2)

# Wendland C2 3-D kernel constants, hdr_kernel.hpp:218-227
KSRH = 1.936492
CEFF0 = 3.342253804929802286e+00
CEFF1 = 1.336901521971920914e+01
ETA_REFERENCE = 1.6

# EOS polytropic index of the ideal-gas closure, hdr_hgas.hpp:767-768
EOS_N = 1.5
GAMMA = 1.0 + 1.0 / EOS_N

# Run parameters written by polytropic_initial_condition/make_and_output_data.hpp:49-54
ALPHA_MAX = 2.0
ALPHA_MIN = 0.1
ALPHU_MAX = 0.0
ALPHU_MIN = 0.0
C_DT = 0.1
DT_MAX = 10.0            # hdr_hgas.hpp:1240
DT_MIN = 1e-16           # hdr_hgas.hpp:1242
