#include <boost/compute/algorithm/sort.hpp>
