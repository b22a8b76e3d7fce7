#include <boost/compute/algorithm/reduce.hpp>
