// dslash_df64.cu -- placeholder until the float-float operator lands.
#include "internal.h"

namespace qg {

struct DArgs;
bool dslash_df64(const DArgs &, bool, int)
{
  set_error("float-float arithmetic is not built");
  return false;
}

}  // namespace qg
