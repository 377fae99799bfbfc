// qmetal/plan.h -- the C++ data model of this library, under the header name a
// client of the reference's C++ API includes (include/qmetal/plan.h there).
// GateKind, Gate, Circuit, PauliString, Hamiltonian, PlanOp, Plan,
// FusionOptions and build_plan live together in one header here.
#pragma once

#include "../../../qmetal_gb300/csrc/circuit.hpp"
