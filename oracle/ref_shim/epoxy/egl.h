/* Stand-in (oracle harness only): no graphics stack is used. */
#pragma once
