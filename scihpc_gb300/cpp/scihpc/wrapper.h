// wrapper.h -- a field with its boundary conditions and links to the shared parameters,
// solvers and scratch (reference scihpc/wrapper.h:14-49).  A velocity wrapper's SLIP normal
// component is treated as NO_SLIP, as the reference's constructors do.
#ifndef SCIHPC_GB300_WRAPPER_H
#define SCIHPC_GB300_WRAPPER_H

#include <string>

#include "bc_factory.h"
#include "dummy_data.h"
#include "global.h"
#include "scalar_data.h"
#include "shared_solvers.h"
#include "vector_data.h"

class wrapper {
public:
    bool is_scalar;
    scalar_data *scalar;
    vector_data *vector;

    wrapper(bool as_scalar, structured_grid *_geo, const bc_info &xlbc_type, const bc_info &xrbc_type);
    wrapper(bool as_scalar, structured_grid *_geo, const bc_info &xlbc_type, const bc_info &xrbc_type,
            const bc_info &ylbc_type, const bc_info &yrbc_type);
    wrapper(bool as_scalar, structured_grid *_geo, const bc_info &xlbc_type, const bc_info &xrbc_type,
            const bc_info &ylbc_type, const bc_info &yrbc_type, const bc_info &zlbc_type, const bc_info &zrbc_type);

    bc_factory *bcFactory;
    bc_factory *bcFactoryU, *bcFactoryV, *bcFactoryW;

    shared_solvers *solvers{};
    problem_parameters *params{};
    dummy_data *dummy{};
    structured_grid *geo;

    void link_solvers(shared_solvers *_solvers);
    void link_params(problem_parameters *_params);
    void link_dummy(dummy_data *_dummy);

    void apply_vel_bc() const;
    void apply_nvel_bc() const;
    void apply_scalar_bc() const;
    void apply_vel_x_bc() const;
    void apply_vel_y_bc() const;
    void apply_vel_z_bc() const;

private:
    void make_factories(const bc_info *b, int nb);
};

#endif
