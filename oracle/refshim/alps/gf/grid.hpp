// Stand-in for ALPSCore's frequency grids (oracle harness only); the linear grid lives in mesh.hpp.
#pragma once
#include "mesh.hpp"
