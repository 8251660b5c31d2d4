// Umbrella header, as the reference's src/atrip.hpp.
#pragma once
#include <atrip/Atrip.hpp>
