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
  int first_outside_quad_local_id() const { return nb_owned + nb_ghosts; }
  int total_local_number_of_outside_quads() const { return nb_outside; }
};
} // namespace kalypsso
