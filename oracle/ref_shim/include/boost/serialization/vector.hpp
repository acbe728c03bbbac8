// The in-process MPI stand-in passes objects by copy, so no serialization is needed.
#ifndef PARS_SHIM_BOOST_SERIALIZATION_VECTOR_HPP
#define PARS_SHIM_BOOST_SERIALIZATION_VECTOR_HPP
#include <vector>
#endif
