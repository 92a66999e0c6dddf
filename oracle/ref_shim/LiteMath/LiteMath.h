#include "../LiteMath.h"
