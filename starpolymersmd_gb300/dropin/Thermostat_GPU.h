// GPU velocity-Verlet integrator for StarPolymersMD: a Thermostat subclass
// constructed like Thermostat_None{box, dt} (star-polymers.cpp:382;
// Thermostat_None.h:8-21) whose propagate runs on the GPU through libsmpc
// (include/smpc.h), sharing the box's device context with the GPU MPC solvent
// (smpc_box.h). Box::Molecules is refreshed on the host by propagate(true),
// the output steps of the driver loop (star-polymers.cpp:466-519).
#ifndef SMPC_DROPIN_THERMOSTAT_GPU_H_
#define SMPC_DROPIN_THERMOSTAT_GPU_H_

#include <string>

#include "Box.h"
#include "Thermostat.h"

class Thermostat_GPU : public Thermostat {
 private:
  double DeltaTHalf;
  static const std::string Name;

 public:
  Thermostat_GPU(Box& box, double dt, bool gaussian = false);
  ~Thermostat_GPU();
  Thermostat_GPU(const Thermostat_GPU&) = delete;
  Thermostat_GPU& operator=(const Thermostat_GPU&) = delete;
  void update_temp();
  void dtime(double& delta_time);
  void propagate(bool calc_epot = false);
  void propagate_gaussian(bool calc_epot = false);
  std::string name() const;
  std::string info() const;
};

#endif  // SMPC_DROPIN_THERMOSTAT_GPU_H_
