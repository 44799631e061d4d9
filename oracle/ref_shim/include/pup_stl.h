/* stand-in: PUP of STL containers is a no-op in the oracle build */
#include "charm++.h"
