// Stand-in header: the exception types live in ptree.hpp of this shim.
#pragma once
#include "ptree.hpp"
