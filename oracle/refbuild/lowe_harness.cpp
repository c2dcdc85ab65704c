// The reference's Lowe_Andersen declares propagate_gaussian
// (Thermostats/Lowe_Andersen.h:24), a pure virtual of Thermostat
// (Thermostats/Thermostat.h:19), but defines it nowhere, so no program can
// construct the class as shipped. Defined here, outside the reference's
// unchanged Lowe_Andersen.cpp, only so the class links; the harness drives
// propagate (Lowe_Andersen.cpp:46-88) and never calls this.
#include "Lowe_Andersen.h"

void Lowe_Andersen::propagate_gaussian(bool calc_epot) { propagate(calc_epot); }
