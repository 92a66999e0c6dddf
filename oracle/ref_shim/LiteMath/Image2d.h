#pragma once
#include "../Image2d.h"
