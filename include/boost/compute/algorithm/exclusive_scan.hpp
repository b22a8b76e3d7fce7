#include <boost/compute/algorithm/scan.hpp>
