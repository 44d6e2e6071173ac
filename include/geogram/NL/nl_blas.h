/*
 * geogram/NL/nl_blas.h -- forwarding header.  Graphite's sources include
 * OpenNL through geogram's header paths (src/lib/OGF/scene_graph/NL/
 * matrix.cpp:40-42, src/lib/OGF/scene_graph/NL/blas.cpp:40,
 * plugins/OGF/WarpDrive/interfaces/mesh_grob_transport_interface.cpp:48,
 * plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.cpp:41,
 * src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:66).  With
 * libnl_gb300's include/ directory first on the include path, every one of
 * those paths resolves to the single header that declares the whole
 * library API.
 */
#include "../../nl.h"
