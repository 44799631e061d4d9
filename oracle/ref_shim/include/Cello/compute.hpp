#include "Cello/cello.hpp"
