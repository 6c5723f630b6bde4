// Stub: the functor bridge runs conforming single blocks; nothing of the AMR hashmap is used.
#pragma once
