/* Stand-in for the configure-generated config.h: the reference build copies src/config-nix.h there (CMakeLists.txt:185). Oracle only. */
#include "config-nix.h"
