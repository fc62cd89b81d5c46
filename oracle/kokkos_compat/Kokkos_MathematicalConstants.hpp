// Host-only stand-in: the reference includes this header but uses none of it.
#pragma once
