// Stand-in for Boost.MPI's environment (see communicator.hpp): nothing to
// initialise in one process.
#pragma once
namespace boost { namespace mpi {
class environment {
  public:
    environment() {}
};
}} // namespace boost::mpi
