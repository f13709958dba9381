// Registers the seir_age system with the engine (one system per
// translation unit so the library compiles in parallel).
#include "engine/factory.cuh"
#include "systems/seir_age.hpp"

DUST2_REGISTER_SYSTEM(dust2gpu::systems::seir_age);
