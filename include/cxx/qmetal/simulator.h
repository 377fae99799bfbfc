// qmetal/simulator.h -- the statevector Simulator for C++ clients, under the
// header name of the reference's C++ API (include/qmetal/simulator.h:30-112
// there): same class, constructor and members, executing on one CUDA
// device. Link against libqmetal.so. kMaxQubits is 34 here (33 there).
#pragma once

#include "../../../qmetal_gb300/csrc/simulator.hpp"
