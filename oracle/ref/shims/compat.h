// Forced include for the reference device-code build: CCCL 3 removed
// thrust::unary_function and thrust::identity, which the reference still names.
#pragma once
#include <thrust/functional.h>
namespace thrust
{
    template<class Arg, class Result> struct unary_function
    {
        using argument_type = Arg;
        using result_type   = Result;
    };
#ifndef SESGB_HAVE_THRUST_IDENTITY
    template<class T> struct identity
    {
        __host__ __device__ const T & operator()( const T & x ) const { return x; }
    };
#endif
} // namespace thrust
