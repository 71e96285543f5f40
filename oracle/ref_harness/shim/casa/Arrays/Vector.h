/* stand-in for casacore's Vector.h: the standard headers the reference's
 * translation units rely on transitively */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <map>
#include <numeric>
#include <string>
#include <vector>
