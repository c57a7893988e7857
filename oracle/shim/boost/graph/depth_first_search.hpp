// Boost-API shim (test infrastructure for oracle/_ref). The reference's test
// utilities include this header but only use their own DFS.
#pragma once
#include "boost/graph/adjacency_list.hpp"
