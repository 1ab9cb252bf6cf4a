/* Stand-in for the OpenCV header that the reference's camera classes include; the
 * frame helpers built by the checker use none of it. */
#pragma once
#include <cstdint>
namespace cv
{
struct Mat
{
    Mat clone() const { return *this; }
};
} // namespace cv
