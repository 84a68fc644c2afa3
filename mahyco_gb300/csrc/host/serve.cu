// Serving loop (continuous batching of hydro runs); filled in below.
#include "runtime.h"

namespace hydro {

struct ServeState {};

void destroy_serve(ServeState* s) { delete s; }

}  // namespace hydro
