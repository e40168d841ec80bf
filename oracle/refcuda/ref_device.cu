// Device half of the reference build: the reference's own CUDA sources,
// included unmodified from the reference checkout (the include path names
// its src/ directory), compiled as one translation unit into a loadable
// device image by oracle/build.py.  Only the files that hold the hot path's
// kernels and the two __constant__ blocks they read are included:
//
//   src/memory_copy.cu  __constant__ Parameter dev_par, Data_Pointer dev_data
//   src/pair.cu         fillFluidCellID, fillSolidCellID, fillVirtCellID,
//                       copyCellList, fillCellList
//   src/fluid.cu        findFluidPair, fluidUpdate (+ the EOS)
//   src/virt.cu         getVirtData
//   src/solid.cu        solidCoupleUpdate, solidDeformationCalculate,
//                       solidForceCalculate, solidUpdate
//
// The kernels take no arguments; the host side (oracle/refcuda/ref_harness.cpp)
// fills the two constant blocks and launches them in the order of
// src/calculation.cu:20-35.  Test infrastructure only.
#include "memory_copy.cu"
#include "pair.cu"
#include "fluid.cu"
#include "virt.cu"
#include "solid.cu"
