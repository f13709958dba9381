// Registers the sirs system, a class written in dust2's own shape and
// adapted by compat/plugin.hpp (one system per translation unit so the
// library compiles in parallel).
#include "engine/factory.cuh"
#include "systems/sirs.hpp"

DUST2_REGISTER_SYSTEM(dust2gpu::systems::sirs);
