// Empty stand-in: the reference includes this header but needs nothing from it.
#pragma once
#include "../Kokkos_Core.hpp"
