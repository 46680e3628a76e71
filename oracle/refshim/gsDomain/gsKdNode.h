// Test-only stand-in: gsAPALMData includes this header but uses nothing from it.
#pragma once
