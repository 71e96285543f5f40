/* empty stand-in */
#pragma once
