// Stand-in for the config.h that kazen_proto's CMake writes from
// src/base/config.h.in, with the reference's default options: no vectorisation
// backend (VECTORIZATION=None selects vec.h's own Vec), and USE_PCG left
// undefined here because the harness draws its inputs itself. TEST
// INFRASTRUCTURE: used only to build the reference-code harness under
// oracle/_ref.
#pragma once
