// Empty stand-in: the FARM reference includes <boost/sort/sort.hpp> in its
// quad-tree header but calls nothing from it.
#pragma once
