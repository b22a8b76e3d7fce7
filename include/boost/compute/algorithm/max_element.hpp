// boost/compute/algorithm/max_element.hpp -- see min_element.hpp.
#ifndef BOOST_COMPUTE_ALGORITHM_MAX_ELEMENT_HPP
#define BOOST_COMPUTE_ALGORITHM_MAX_ELEMENT_HPP
#include <boost/compute/algorithm/min_element.hpp>
#endif
