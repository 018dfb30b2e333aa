// Stand-in for allscale/utils/static_grid.h: included by cell.h:12 but no
// symbol from it is used on the path. TEST INFRASTRUCTURE ONLY (oracle).
#pragma once
