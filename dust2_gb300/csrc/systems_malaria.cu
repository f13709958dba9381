// Registers the mixed-time malaria system with the engine (one system per
// translation unit so the library compiles in parallel).
#include "engine/factory.cuh"
#include "systems/malaria.hpp"

DUST2_REGISTER_SYSTEM(dust2gpu::systems::malaria);
