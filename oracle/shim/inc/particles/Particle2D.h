// Case shim: the reference includes "../../particles/Particle2D.h" while the
// file on disk is particles/particle2D.h.  The -I path that ends in
// shim/inc/a/b makes that relative include land here.
#pragma once
#include <particles/particle2D.h>
