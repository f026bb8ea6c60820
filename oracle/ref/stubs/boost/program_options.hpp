// Only the type name is needed: the oracle build fills InputParameters directly.
#pragma once
namespace boost { namespace program_options { class variables_map {}; } }
