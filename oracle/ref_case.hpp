// The 20x20x4 three-phase waterflood of the golden vectors and the trajectory check (test infrastructure).
//
// Built from the reference's own input generators (generateGeometry / generateRock / makeCorrelationPVT /
// makeCoreySWOF / makeCoreySGOF, engine/src/tools.cpp:13-245) on top of the demo case, which supplies fluids in
// place, equilibration and controls: 100 x 100 x 20 ft cells, log-normal permeability (ln 100 mD, sigma 1,
// correlation 5 x 5 cells, seed 0), porosity 0.2, Corey exponents 2 with Swc = Sor = 0.2, a water injector at
// (0,0) and a producer at (nx-1, ny-1), both perforated in every layer.
#pragma once
#include "ressim/case.h"
#include "ressim/tools.h"

namespace rsgref {

inline ressim::Case waterfloodCase(int nsteps, double stepDays, int linearSolver, int nx = 20, int ny = 20, int nz = 4,
                                   double sigma = 1.0, unsigned seed = 0u) {
    using namespace ressim;
    Case c = makeDemoCase();
    c.title = "generated waterflood";
    GeomInput gi; gi.nx = nx; gi.ny = ny; gi.nz = nz; gi.dx = 100; gi.dy = 100; gi.dz.assign(size_t(nz), 20.0); gi.top = 8325;
    c.grid = GridInput{};
    generateGeometry(gi, c.grid);
    RockGenInput ri; ri.layerPerm = {100}; ri.layerPoro = {0.2}; ri.sigmaLn = sigma; ri.corrX = 5; ri.corrY = 5;
    ri.poroPermExp = 0; ri.seed = seed;
    generateRock(ri, c.grid);
    CorrelationInput pvt;
    makeCorrelationPVT(pvt, c.units, c.props);
    CoreyInput cor; cor.swc = 0.2; cor.sorw = 0.2; cor.nw = 2; cor.now = 2;
    makeCoreySWOF(cor, c.props.swof);
    makeCoreySGOF(cor, c.props.sgof);
    c.wells.clear();
    WellInput prod; prod.name = "PROD"; prod.type = WellType::Producer; prod.i = nx - 1; prod.j = ny - 1;
    { Completion cp; cp.i = nx - 1; cp.j = ny - 1; cp.k1 = 0; cp.k2 = nz - 1; prod.completions.push_back(cp); }
    WellInput inj; inj.name = "INJ"; inj.type = WellType::WaterInjector; inj.i = 0; inj.j = 0;
    { Completion cp; cp.i = 0; cp.j = 0; cp.k1 = 0; cp.k2 = nz - 1; inj.completions.push_back(cp); }
    c.wells = {prod, inj};
    WellControl wp; wp.well = "PROD"; wp.mode = Control::ORAT; wp.orat = 1500; wp.bhp = 1000;
    WellControl wi; wi.well = "INJ"; wi.mode = Control::RATE; wi.rate = 2000; wi.bhp = 6000;
    c.schedule.clear();
    for (int s = 0; s < nsteps; ++s) {
        ReportStep r; r.length = stepDays;
        if (s == 0) r.controls = {wp, wi};
        c.schedule.push_back(r);
    }
    c.tuning.linearSolver = linearSolver;
    c.tuning.blockSolver = true;
    return c;
}

}  // namespace rsgref
