// Stub: the functor bridge runs conforming single blocks; nothing of the face status is used.
#pragma once
