// ressim/blocksolve.h -- the header tools/lsbench.cpp:3 includes but the reference tree does not ship.
// Supplies BlockSolver / BlockSolverOptions / BlockSolverStats (tools/lsbench.cpp:65-81) over the GB300 solver
// (include/rsg_ressim_adapter.hpp) and a no-op accelerator registry (app/src/gpu_solver.cpp:350-353 registers a
// D3D11 one, a graphics path that is not part of this build).
#pragma once
#include "rsg_ressim_adapter.hpp"

namespace ressim {
using BlockSolverOptions = rsg::BlockSolverOptions;
using BlockSolverStats = rsg::BlockSolverStats;
using BlockSolver = rsg::RsgBlockSolver;
class BlockAccelerator {
public:
    virtual ~BlockAccelerator() = default;
    virtual const char* name() const = 0;
    virtual bool setup(int nCells, int nb, const std::vector<int>& rp, const std::vector<int>& ci, const std::vector<double>& blocks) = 0;
    virtual bool apply(const double* r, double* z) = 0;
};
inline BlockAccelerator*& blockAcceleratorSlot() { static BlockAccelerator* a = nullptr; return a; }
inline void setBlockAccelerator(BlockAccelerator* a) { blockAcceleratorSlot() = a; }
inline BlockAccelerator* blockAccelerator() { return blockAcceleratorSlot(); }
}  // namespace ressim
