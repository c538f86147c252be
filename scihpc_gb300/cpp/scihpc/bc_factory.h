// bc_factory.h -- boundary-condition names and per-face configuration (reference
// scihpc/bc_factory.h:13-59: the kinds are strings, bc_info{NEUMANN} etc.).  The fills run
// on the GPU through scihpc_bc_fill; periodic, Neumann, no-slip, slip and Dirichlet faces
// follow the reference's fills (periodic.cpp, neumann.cpp, no_slip.cpp, slip.cpp,
// dirichlet.cpp).
#ifndef SCIHPC_GB300_BC_FACTORY_H
#define SCIHPC_GB300_BC_FACTORY_H

#include <string>

#include "global.h"
#include "structured_grid.h"
#include "vector_data.h"

const std::string NO_SLIP = "no_slip";
const std::string SLIP = "slip";
const std::string PERIODIC = "periodic";
const std::string NEUMANN = "neumann";
const std::string DIRICHLET = "dirichlet";

struct bc_info {
    std::string type = "NoSlip";
    DataType value = 0.0;
};

class bc_factory {
public:
    bc_factory(structured_grid *geo, const bc_info &xl_bc, const bc_info &xr_bc);
    bc_factory(structured_grid *geo, const bc_info &xl_bc, const bc_info &xr_bc, const bc_info &yl_bc,
               const bc_info &yr_bc);
    bc_factory(structured_grid *geo, const bc_info &xl_bc, const bc_info &xr_bc, const bc_info &yl_bc,
               const bc_info &yr_bc, const bc_info &zl_bc, const bc_info &zr_bc);

    bc_info xlbc, xrbc, ylbc, yrbc, zlbc, zrbc;
    DataType dx, dy, dz;
    structured_grid *geo;

    // fills of one field in place on the GPU: cell centred, or staggered in x / y / z
    void apply_node_centered(scalar_data *f);
    void apply_node_staggered_x(scalar_data *f);
    void apply_node_staggered_y(scalar_data *f);
    void apply_node_staggered_z(scalar_data *f);

    // boundary codes of the C ABI (0 periodic, 1 neumann, 2 no_slip, 3 slip, 4 dirichlet)
    // in the order xl, xr, yl, yr, zl, zr
    void codes(int types[6], double values[6]) const;
};

#endif
