// boost/compute.hpp -- the whole drop-in layer (the reference's umbrella
// header, include/boost/compute.hpp).
#ifndef BOOST_COMPUTE_HPP
#define BOOST_COMPUTE_HPP
#include <boost/compute/algorithm.hpp>
#include <boost/compute/async/future.hpp>
#include <boost/compute/async/wait.hpp>
#include <boost/compute/container/vector.hpp>
#include <boost/compute/core.hpp>
#include <boost/compute/event.hpp>
#include <boost/compute/functional.hpp>
#include <boost/compute/iterator/buffer_iterator.hpp>
#include <boost/compute/iterator/counting_iterator.hpp>
#include <boost/compute/iterator/discard_iterator.hpp>
#include <boost/compute/iterator/transform_iterator.hpp>
#include <boost/compute/function.hpp>
#include <boost/compute/lambda.hpp>
#endif
