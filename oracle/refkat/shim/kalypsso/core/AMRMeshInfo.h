// Stub of kalypsso-core's mesh counts for the functor bridge: owned blocks first, no MPI ghosts,
// outside blocks after them.
#pragma once
namespace kalypsso
{
struct AMRMeshInfo
{
  int nb_owned = 1, nb_ghosts = 0, nb_outside = 0;
  int local_num_quadrants() const { return nb_owned; }
  int local_num_ghosts() const { return nb_ghosts; }
  int local_num_mirrors() const { return 0; }
};
} // namespace kalypsso
