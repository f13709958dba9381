// Registers the sir system with the engine (one system per
// translation unit so the library compiles in parallel).
#include "engine/factory.cuh"
#include "systems/sir.hpp"

DUST2_REGISTER_SYSTEM(dust2gpu::systems::sir);
