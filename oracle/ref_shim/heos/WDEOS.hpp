// heos/WDEOS.hpp — type-only stand-in for the white-dwarf EOS library that the
// reference's hdr_heos.hpp includes but does not ship.  TEST INFRASTRUCTURE:
// it lets oracle/ref_glue.cpp compile hdr_hgas.hpp from the reference tree.
// Only the damping and Helmholtz paths call these members; the ideal-gas
// step glue that ref_glue.cpp binds (EOS, time step, energy, predictor,
// corrector, alpha derivative) never does.  They return 0.
#pragma once

namespace OTOO {
struct EOS {
    virtual ~EOS() {}
    virtual double GetP(double, double) { return 0.0; }
    virtual double GetT(double, double) { return 0.0; }
    virtual double GetS(double, double) { return 0.0; }
    virtual double GetE(double, double) { return 0.0; }
    virtual double GetEmin2(double) { return 0.0; }
};
struct WDEOSforDumping : EOS {
    WDEOSforDumping(double, double, double, double, double) {}
};
}  // namespace OTOO
