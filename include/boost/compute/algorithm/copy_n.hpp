#include <boost/compute/algorithm/copy.hpp>
