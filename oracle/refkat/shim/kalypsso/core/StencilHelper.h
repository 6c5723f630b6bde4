// Stub of kalypsso-core's stencil helper for the functor bridge: the face-side tag only.
#pragma once
namespace kalypsso
{
enum class face_type_t : int
{
  LEFT = 0,
  RIGHT = 1
};
} // namespace kalypsso
