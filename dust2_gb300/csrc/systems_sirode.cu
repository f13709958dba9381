// Registers the sirode system with the engine (one system per
// translation unit so the library compiles in parallel).
#include "engine/factory.cuh"
#include "systems/sirode.hpp"

DUST2_REGISTER_SYSTEM(dust2gpu::systems::sirode);
