// Stand-in for ALPSCore's config header (oracle harness only): nothing is needed.
#pragma once
