// GPU MPC solvent for StarPolymersMD: a drop-in for
// star-polymers/lib/Hydrodynamics/MPC.h with the same class name, constructor
// and public methods (MPC.h:25-120), implemented over the C ABI of libsmpc
// (include/smpc.h). Put this directory before lib/Hydrodynamics on the include
// path and compile MPC_gpu.cpp + smpc_box.cpp (and link libsmpc) instead of
// lib/Hydrodynamics/MPC.cpp: star-polymers.cpp, mpc_test.cpp and VelocityX
// compile unchanged.
//
// The solvent lives on the GPU. `Fluid` and the cell lists are a host mirror,
// refreshed from the device when a host-side reader needs them (print_fluid*,
// operator(), unitary, the per-cell getters). MPC::step draws its random
// numbers from the reference's own Rand stream in the reference's order (grid
// shift, then per cell the gamma variate and the two axis uniforms), so a run
// follows the CPU reference's trajectory to FP64 round-off. The monomers are
// shared with the integrator through one device context per Box
// (smpc_box.h): with Thermostat_GPU they stay on the device; with a CPU
// thermostat each collision uploads them and writes the collided state back.
#ifndef SMPC_DROPIN_MPC_H_
#define SMPC_DROPIN_MPC_H_

#include <array>
#include <csignal>
#include <cmath>
#include <fstream>
#include <iostream>
#include <vector>

#include "Analysis.h"
#include "Functions.h"
#include "Hydrodynamics.h"
#include "Molecule.h"
#include "Particle.h"
#include "Rand.h"

class Box;
class MPC : public Hydrodynamics {
  friend class Box;
  friend class VelocityX;

 protected:
  double Temperature;
  double Shear;
  unsigned step_update;
  unsigned NumberOfCells;
  unsigned NumberOfMPCParticles;
  double c;
  double s;
  double delrx;
  bool shear_on;
  bool angular_momentum;
  std::array<int, 3> BoxSize;
  // host mirror of the last sort (MPC.h:40-41), rebuilt on demand
  mutable std::vector<std::vector<MPCParticle*>> MPCCellList;
  mutable std::vector<unsigned> MPCCellListFluidParticles;

  // device bookkeeping
  bool fluid_dirty = true;          // host Fluid is newer than the device copy
  mutable bool host_stale = false;  // device is newer than Fluid / MPCCellList
  bool collided = false;            // a collision has run (cell lists exist)
  std::vector<unsigned> cell_total;
  std::vector<double> draw_gamma, draw_phi, draw_theta;
  void pull() const;
  [[noreturn]] void on_device(const char* what) const;

 public:
  mutable std::vector<MPCParticle> Fluid;
  MPC(Box&, double, int N_c, double aShear = 0., unsigned step = 1, bool angular_mom = false);
  ~MPC();
  MPC(const MPC&) = delete;
  MPC& operator=(const MPC&) = delete;

  void initialize();
  void initialize(string filename, std::array<int, 3> Box_old);

  // MPC routine:
  void step(const long int& t, const double& dt);
  void streaming(const double& dt);
  void sort();
  void sort(std::vector<std::vector<MPCParticle*>>&);
  void collide(unsigned, const Vector3d&);
  void collide(const std::vector<MPCParticle*>& List, const Vector3d& CMV);
  void thermostat(unsigned i, const Vector3d& CMV);
  void thermostat(const std::vector<MPCParticle*>&, const Vector3d&);
  void periodic_image_box(unsigned);
  void undo_periodic_image_box(unsigned);
  void check_bounds();
  void shiftParticles(const Vector3d& Shift);
  void LEBC(Particle&);
  void LEBC(Vector3d&, Vector3d&);
  Vector3d& wrap(Vector3d&);
  Vector3d wrap(Vector3d&&);
  void wrap(Particle&);
  void wrap(Vector3d&, Vector3d&);

  void LEBC_to_zero(Vector3d&, Vector3d&);
  Vector3d& wrap_to_zero(Vector3d&);
  void wrap_to_zero(Vector3d&, Vector3d&);
  void wrap_to_zero(Particle&);

  Vector3d relative_position(Particle& one, Particle& two);
  Vector3d relative_position(const Vector3d, const Vector3d);

  // getter methods:
  void calculateCMV(unsigned Index, Vector3d&);
  void calculateCMV(std::vector<MPCParticle*>& List, Vector3d& CMV);
  void calculateFluidVelocity(unsigned Index, Vector3d&);
  void calculateCMP(unsigned Index, Vector3d&);
  void calculateAngular(unsigned Index, Vector3d& Angular, const Vector3d& CMV,
                        const Vector3d& CMP, const Matrix3d& Rotation);
  void calculateAngularMomentum(unsigned Index, Vector3d&, const Vector3d& CMV, const Vector3d& CMP);
  double calculateEkinInCell(unsigned Index);
  double calculateEkinTotal();
  double calculateCurrentTemperature();
  unsigned filledCells();
  unsigned NumberOfParticles() const { return NumberOfMPCParticles; }

  template <class UnitaryFunc>
  UnitaryFunc unitary(UnitaryFunc& func) const {
    pull();
    return for_each(Fluid.cbegin(), Fluid.cend(), func);
  }

  template <class UnaryFunc, class BinaryFunc>
  void operator()(UnaryFunc& ufunc, BinaryFunc& bfunc) const {
    pull();
    for (auto first = Fluid.cbegin(); first != Fluid.cend(); ++first) {
      ufunc(*first);
      for (auto second = first + 1; second != Fluid.cend(); ++second) bfunc(*first, *second);
    }
  }

  template <class UnaryFunc>
  void operator()(UnaryFunc& ufunc) const {
    pull();
    for (auto it = Fluid.cbegin(); it != Fluid.cend(); ++it) ufunc(*it);
  }

  void print_fluid(FILE*, int, int, int);
  void print_fluid_with_coordinates(FILE*, int, int, int);
  void print_fluid_complete(FILE*);
};

#endif  // SMPC_DROPIN_MPC_H_
