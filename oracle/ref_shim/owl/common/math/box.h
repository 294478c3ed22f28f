// Forwards to the host stand-ins of the reference's unvendored dependencies
// (test infrastructure; see aloha_owl_shim.h).
#pragma once
#include "aloha_owl_shim.h"
